"""Edge cases of the render entry points on the GPU.

- Ragged and degenerate frames (1x1, a single row or column, sizes that are
  no multiple of the 16x8 tile or of the 8x4 persistent tile) render every
  pixel and agree with the oracle's FP64 twin at the parity tolerance
  (radiance p99 <= 1e-5), for both schedules.
- The smallest gas grids (one radial cell, an azimuth of one or two cells that
  wraps onto itself, one vertical cell) render in FP32 and agree with the
  oracle's FP64 twin (radiance median <= 1e-4, class mismatches <= 1 %): the
  float sampler's index math at its limits.
- Arguments the reference rejects come back as ST_EINVAL without touching
  the device: sizes <= 0 or beyond 2^30 pixels, samples <= 0, dt <= 0,
  |a| > M (src/gr.jl:31), an unknown integrator order; and a gas grid of
  2^31 cells or more (the float sampler indexes the grid in 32 bits), which
  is refused before its density pointer is read.
"""
import ctypes as C
import types

import numpy as np
import pytest

from oracle import oracle as O
from spacetime_gb300 import _abi, workloads
from spacetime_gb300.api import Context, Kerr

from .helpers import compare, gpu_render, oracle_scene

pytestmark = pytest.mark.gpu

FP64 = _abi.ST_PREC_FP64


@pytest.fixture(scope="module")
def sky():
    return workloads.sky(512, 256)


def _draft_disc():
    w = workloads.config0()
    w.semantics = _abi.ST_SEM_DRAFT
    w.emitter = _abi.ST_EMIT_KS_EXACT
    w.params = dict(samples=1, pixel_jitter=0, exit_landing=1)
    return w


@pytest.mark.parametrize("size", [(1, 1), (1, 9), (17, 1), (17, 3), (33, 27)])
@pytest.mark.parametrize("schedule", [_abi.ST_SCHED_PIXEL, _abi.ST_SCHED_PERSISTENT])
def test_ragged_frames_match_the_twin(built_lib, sky, size, schedule):
    w = _draft_disc().scaled(*size)
    g = gpu_render(w, sky, FP64, schedule=schedule)
    assert g.image.shape == (size[1], size[0], 3)
    assert np.isfinite(g.image).all()
    assert g.stats["rays"] == size[0] * size[1]
    ref, rays = oracle_scene(w, sky, O.INT_RK4).render()
    c = compare(g.image, g.diag, ref, rays)
    assert c["class_mismatch"] == 0, c
    assert c["rad_p99"] <= 1e-5, c


def test_arguments_the_reference_rejects(built_lib, sky):
    w = _draft_disc().scaled(8, 8)
    with Context(sky, disc=w.disc, emitter=w.emitter) as ctx:
        def code(bh=w.bh, **kw):
            args = dict(width=8, height=8)
            args.update(kw)
            p = ctx.params(_abi.ST_SEM_DRAFT, **args)
            # a one-pixel host buffer: the library validates before it writes
            with pytest.raises(_abi.StError) as e:
                ctx.render_raw(w.cam, bh, p, out=np.empty((1, 1, 3), np.float32))
            return e.value.code
        assert code(width=0) == _abi.ST_EINVAL
        assert code(height=-3) == _abi.ST_EINVAL
        assert code(width=1 << 16, height=1 << 15) == _abi.ST_EINVAL   # 2^31 pixels
        assert code(samples=0) == _abi.ST_EINVAL
        assert code(dt=0.0) == _abi.ST_EINVAL
        assert code(order=5) == _abi.ST_EINVAL
        assert code(bh=types.SimpleNamespace(M=1.0, a=1.5)) == _abi.ST_EINVAL   # past the C ABI
        with pytest.raises(ValueError):
            Kerr(1.0, 1.5)                                                    # and in the Python API
        # a gas grid of 2^31 cells: refused before the (one-cell) buffer is read
        cell = np.zeros(1, np.float32)
        big = _abi.StVolume(cell.ctypes.data_as(C.POINTER(C.c_float)), 1 << 16, 1 << 10, 1 << 5,
                            1.0, 3.0, 1.0, 1.0, 1.0, 2)
        assert ctx._lib.st_context_set_volume(ctx._h, C.byref(big)) == _abi.ST_EINVAL
        # the context is still usable afterwards
        ok = ctx.render_raw(w.cam, w.bh, ctx.params(_abi.ST_SEM_DRAFT, width=8, height=8))
        assert np.isfinite(ok.image).all()


def test_captured_rays_finish_at_launch_without_matter(built_lib, sky):
    """With neither disc nor gas, a ray the Bardeen launch test proves captured
    is black whatever its integration does and collects nothing, so the kernel
    finishes it at launch: its pixel is black with zero steps, and the frame
    still matches the FP64 twin (which integrates every ray) at the parity
    tolerance."""
    w = workloads.config1_nogas().scaled(96, 54)
    w.params = dict(samples=1, pixel_jitter=0, exit_landing=1)
    g = gpu_render(w, sky, FP64)
    bcapt = (g.diag["flags"] & _abi.ST_RAY_BCAPT) > 0
    assert bcapt.sum() > 100
    assert np.all(g.diag["steps"][bcapt] == 0)
    assert np.all(g.image[bcapt] == 0.0)
    ref, rays = oracle_scene(w, sky, O.INT_RK4).render()
    assert np.all(rays["steps"][bcapt] > 0)            # the twin integrates them
    c = compare(g.image, g.diag, ref, rays)
    assert c["class_mismatch"] == 0, c
    assert c["dir_median"] <= 1e-9 and c["rad_p99"] <= 1e-5, c


@pytest.mark.parametrize("shape", [(2, 1, 2), (3, 2, 3), (5, 3, 2)])
def test_smallest_gas_grids_fp32(built_lib, sky, shape):
    nr, nphi, nz = shape
    w = workloads.config1().scaled(128, 72)
    w.vol = workloads.volume(nr, nphi, nz, 2.32, 25.0, 0.05)
    g = gpu_render(w, sky, _abi.ST_PREC_FP32)
    assert g.stats["gas_samples"] > 0
    assert np.isfinite(g.image).all()
    ref, rays = oracle_scene(w, sky, O.INT_RK4).render()
    c = compare(g.image, g.diag, ref, rays)
    print(shape, c)
    assert c["class_mismatch"] <= 0.01 * c["n"], c
    assert c["rad_median"] <= 1e-4, c   # measured 0.6e-6 .. 3e-6



@pytest.mark.parametrize("prec", [_abi.ST_PREC_FP64, _abi.ST_PREC_FP32])
def test_non_finite_rays_end_black(built_lib, prec):
    """The NaN guard (src/metal.jl:1414-1421): a ray whose state stops being
    finite is captured and painted black, as the reference does, instead of
    running to its step budget.  A NaN field of view (fov_factor) makes every
    ray of the frame non-finite from launch (the host does not reject it, as
    the reference's camera block does not): each ray takes one step, is caught
    by the guard and ends black, the launch finishes with status OK, and the
    oracle's twin (which restates the same guard) agrees."""
    w = workloads.config1_thin().scaled(32, 18)
    w.params = dict(samples=1, pixel_jitter=0, exit_landing=1)
    w.cam.fov_factor = float("nan")
    sky = workloads.sky(512, 256)
    g = gpu_render(w, sky, prec)
    assert g.stats["status"] == _abi.ST_OK and g.stats["rays"] == 32 * 18
    assert g.stats["steps"] == 32 * 18          # one step each: the guard stops them
    assert (g.image == 0).all()
    assert ((g.diag["flags"] & _abi.ST_RAY_CAPTURED) > 0).all()
    assert ((g.diag["flags"] & _abi.ST_RAY_BLACK) > 0).all()
    ref, rays = oracle_scene(w, sky, O.INT_RK4).render()
    assert (ref == 0).all() and ((rays["flags"] & O.RAY_BLACK) > 0).all()
