"""The CPU side of bench.py, on the CPU.

bench.py's CPU baseline (and its reference arm) times the oracle on a strided
sample of the benchmarked frame's own pixels, launched through
Scene.trace_dirs from camera-frame directions that bench._strided_dirs builds
the way the pinhole camera maps pixel centres.  At stride 1 those directions
are every pixel of the frame in row order, so the rays they trace must be
the rays the oracle's own pixel path renders, record for record; a stride
keeps the pixels on its grid.
"""
import numpy as np

import bench
from oracle import oracle as O
from spacetime_gb300 import workloads

W, H = 48, 27


def test_strided_sample_traces_the_frames_own_rays():
    w = workloads.config1_nogas().scaled(W, H)
    sky = workloads.sky(256, 128)
    sc = O.scene_for(w, sky, O.INT_RK4)
    _, rays = sc.render()
    dirs, stride = bench._strided_dirs(w, W, H, W * H)
    assert stride == 1 and dirs.shape == (W * H, 3)
    np.testing.assert_allclose(np.linalg.norm(dirs, axis=1), 1.0, rtol=1e-15)
    got = sc.trace_dirs(dirs)
    ref = rays.reshape(-1)
    np.testing.assert_array_equal(got["flags"], ref["flags"])
    np.testing.assert_array_equal(got["steps"], ref["steps"])
    np.testing.assert_allclose(got["dir"], ref["dir"], rtol=0, atol=1e-12)


def test_strided_sample_keeps_its_grid():
    w = workloads.config1_nogas().scaled(W, H)
    dirs, stride = bench._strided_dirs(w, W, H, (W * H) // 9)
    assert stride == 3
    full, _ = bench._strided_dirs(w, W, H, W * H)
    grid = full.reshape(H, W, 3)[1::3, 1::3].reshape(-1, 3)
    np.testing.assert_array_equal(dirs, grid)
