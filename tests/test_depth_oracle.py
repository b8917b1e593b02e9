"""Depth buckets in the oracle (render_depth_mtl, src/metal.jl:1935-1990;
bucketing at :1170-1175, 1425-1426, 1489-1497, 1556-1563, 1687-1690).

- The buckets of one pass sum to the plain pass: bucketing only moves
  emission between channels (float32 outputs, rtol 1e-6).
- With neither disc nor gas every channel but the last (the sky) is zero.
- Known answer: a camera 30 M above a face-on disc (6-20 M) sees the disc's
  direct image along paths of 30.6-36.1 M; with 10 buckets,
  trunc((ln ell - ln 1.5) 8 / ln 80) + 1 = 6 for that whole range, so the
  direct image lands in bucket 6 (index 5).
"""
import numpy as np
import pytest

from oracle import oracle as O
from spacetime_gb300 import workloads
from spacetime_gb300.scene import Camera


@pytest.fixture(scope="module")
def sky():
    return workloads.sky(256, 128)


def _pair(scene, nb):
    img, rays = scene.render()
    bk = scene.render_depth(nb)
    return img, rays, bk


@pytest.mark.parametrize("case", ["schw_disc", "kerr_gas"])
def test_buckets_sum_to_the_plain_pass(sky, case):
    if case == "schw_disc":
        w = workloads.config0().scaled(48, 27)
        w.semantics = 1
        w.emitter = 1
        w.params = dict(samples=1, pixel_jitter=0, exit_landing=0)
    else:
        w = workloads.config1().scaled(40, 24)
    s = O.scene_for(w, sky, O.INT_RK4)
    img, rays, bk = _pair(s, 10)
    assert bk.shape == (w.height, w.width, 10, 3)
    np.testing.assert_allclose(bk.astype(np.float64).sum(axis=2), img, rtol=1e-6, atol=1e-9)
    emis = bk[:, :, :-1, :].sum(axis=(2, 3))
    assert (emis > 0).sum() > 0.05 * w.width * w.height   # the disc / gas shows up
    # black pixels carry no sky; escaped pixels' sky bucket is non-negative
    black = (rays["flags"] & O.RAY_BLACK) > 0
    assert np.all(bk[black][:, -1, :] == 0.0)
    assert np.all(bk >= 0.0)


def test_sky_only_fills_the_last_bucket(sky):
    w = workloads.config0().scaled(32, 18)
    w.semantics = 1
    w.disc = None
    w.params = dict(samples=1, pixel_jitter=0, exit_landing=0)
    s = O.scene_for(w, sky, O.INT_RK4)
    img, _, bk = _pair(s, 4)
    assert np.all(bk[:, :, :-1, :] == 0.0)
    np.testing.assert_allclose(bk[:, :, -1, :], img, rtol=1e-6, atol=1e-9)


def test_face_on_disc_lands_in_the_path_length_bucket(sky):
    cam = Camera.look_at((0.0, 0.0, 30.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), fov_factor=0.75)
    s = O.Scene(cam=cam, M=1.0, a=0.0, sky=sky, width=48, height=48, semantics=O.SEM_DRAFT,
                integrator=O.INT_RK4, disc=dict(inner=6.0, outer=20.0), emitter=O.EMIT_KS_EXACT,
                exit_landing=0)
    img, rays, bk = _pair(s, 10)
    hit = (rays["r_cross"] > 6.5) & (rays["r_cross"] < 19.5)
    assert hit.sum() > 200
    emis = bk[hit][:, :-1, :].sum(axis=2)                  # (pixels, 9) emission per bucket
    tot = emis.sum(axis=1)
    assert np.all(tot > 0)
    assert np.all(emis[:, 5] >= 0.99 * tot), np.unique(np.argmax(emis, axis=1), return_counts=True)


def test_bucket_count_below_three_is_rejected(sky):
    w = workloads.config0().scaled(8, 8)
    w.semantics = 1
    s = O.scene_for(w, sky, O.INT_RK4)
    with pytest.raises(RuntimeError):
        s.render_depth(2)
