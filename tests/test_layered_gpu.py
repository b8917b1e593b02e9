"""The layered engine on the GPU (update_sky_fan!, render_layered_gpu!,
src/metal.jl:2394-3147), Schwarzschild, kernel rules.

- Fan: every entry (coarse over psi in [0, pi], fine across the band) against
  the oracle's FP64 twin of the same ray (orc_trace_dirs): escape flag
  identical, exit angle within 1e-6 rad (the fan stores float32).
- Sky: the fan-driven frame against the full per-pixel trace of the same
  frame: exit directions (interpolated in psi) median <= 1e-6 rad, p99 <= 1e-4.
- With a disc: the layer pass plus composite against the full trace:
  radiance median <= 1e-4, and at half layer resolution the frame stays close
  while tracing fewer steps.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from spacetime_gb300 import _abi, workloads
from spacetime_gb300.api import Context
from spacetime_gb300.scene import Camera

from .helpers import angle, gpu_render

pytestmark = pytest.mark.gpu

FP64, FP32 = _abi.ST_PREC_FP64, _abi.ST_PREC_FP32


def _scene(disc=False, w=192, h=108):
    wl = workloads.config0().scaled(w, h)
    wl.semantics = _abi.ST_SEM_DRAFT
    wl.emitter = _abi.ST_EMIT_KS_EXACT
    wl.params = dict(samples=1, pixel_jitter=0, exit_landing=1)
    if not disc:
        wl.disc = None
    return wl


def _params(ctx, wl, prec=FP64, **kw):
    return ctx.params(wl.semantics, width=wl.width, height=wl.height, precision=prec, **wl.params, **kw)


def test_fan_fp64_vs_oracle_twin(built_lib):
    wl = _scene()
    sky = workloads.sky(512, 256)
    with Context(sky, disc=None, emitter=wl.emitter) as ctx:
        fan, fine, band = ctx.sky_fan(wl.cam, wl.bh, _params(ctx, wl))
    r = float(np.linalg.norm(wl.cam.pos))
    fcam = Camera(np.array([r, 0.0, 0.0]), np.array([1.0, 0, 0]), np.array([0, 1.0, 0]), np.array([0, 0, 1.0]),
                  1.0, np.zeros(3))
    one = workloads.Workload("fan", wl.bh, fcam, 4, 4, _abi.ST_SEM_DRAFT, None, wl.emitter,
                             params=dict(samples=1, pixel_jitter=0, exit_landing=1))
    sc = O.scene_for(one, workloads.sky(64, 32), O.INT_RK4)
    n, nf = fan.shape[0], fine.shape[0]
    psi = math.pi * np.arange(n) / (n - 1)
    lo, hi = float(band[0]), float(band[1])
    assert 0.0 < lo < hi < math.pi
    psif = lo + (hi - lo) * np.arange(nf) / (nf - 1)
    for ang, tab in ((psi, fan), (psif, fine)):
        rays = sc.trace_dirs(np.stack([np.cos(ang), np.sin(ang), np.zeros_like(ang)], 1))
        esc = (rays["flags"] & O.RAY_BLACK) == 0
        assert np.array_equal(esc, tab[:, 0] > 0.5)
        d = rays["dir"][esc][:, :2]
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        g = tab[esc][:, 1:3].astype(np.float64)
        g /= np.linalg.norm(g, axis=1, keepdims=True)
        err = np.abs(np.arctan2(d[:, 0] * g[:, 1] - d[:, 1] * g[:, 0], (d * g).sum(1)))
        assert err.max() <= 1e-6, err.max()
    # the band brackets the coarse fan's single escape/capture transition
    flips = np.nonzero(fan[1:, 0] != fan[:-1, 0])[0]
    assert flips.size == 1 and lo <= psi[flips[0]] and psi[flips[0] + 1] <= hi


def test_fan_sky_matches_full_trace(built_lib):
    wl = _scene()
    sky = workloads.sky(512, 256)
    with Context(sky, disc=None, emitter=wl.emitter) as ctx:
        lay = ctx.render_layered_raw(wl.cam, wl.bh, _params(ctx, wl), diag=True)
        full = ctx.render_raw(wl.cam, wl.bh, _params(ctx, wl), diag=True)
    ge = (lay.diag["flags"] & _abi.ST_RAY_ESCAPED) > 0
    fe = (full.diag["flags"] & _abi.ST_RAY_ESCAPED) > 0
    assert (ge != fe).mean() <= 0.005
    both = ge & fe
    d = angle(lay.diag["dir"][both], full.diag["dir"][both])
    print("fan sky vs trace: median", np.median(d), "p99", np.percentile(d, 99), "max", d.max(),
          "ms", lay.stats["kernel_ms"], full.stats["kernel_ms"])
    assert np.median(d) <= 1e-6 and np.percentile(d, 99) <= 1e-4
    assert np.isfinite(lay.image).all()


@pytest.mark.parametrize("prec", [FP64, FP32])
def test_layer_and_composite_match_full_trace(built_lib, prec):
    wl = _scene(disc=True)
    sky = workloads.sky(512, 256)
    with Context(sky, disc=wl.disc, emitter=wl.emitter) as ctx:
        lay = ctx.render_layered_raw(wl.cam, wl.bh, _params(ctx, wl, prec))
        half = ctx.render_layered_raw(wl.cam, wl.bh, _params(ctx, wl, prec), layer_size=(wl.width // 2, wl.height // 2))
        full = ctx.render_raw(wl.cam, wl.bh, _params(ctx, wl, prec))
    lum = full.image.astype(np.float64).sum(-1)
    rel = np.abs(lay.image - full.image).sum(-1) / np.maximum(lum, 1e-6)
    relh = np.abs(half.image - full.image).sum(-1) / np.maximum(lum, 1e-6)
    print("layered vs trace: median", np.median(rel), "p99", np.percentile(rel, 99),
          "half-res layer median", np.median(relh), "steps", lay.stats["steps"], half.stats["steps"],
          full.stats["steps"], "ms", lay.stats["kernel_ms"], half.stats["kernel_ms"], full.stats["kernel_ms"])
    assert lay.stats["status"] == _abi.ST_OK
    assert np.median(rel) <= 1e-4
    # rays the fan proves miss the disc are not traced
    assert lay.stats["steps"] < full.stats["steps"]
    assert half.stats["steps"] < lay.stats["steps"]
    assert np.median(relh) <= 0.05 and np.isfinite(half.image).all()


def test_layered_rejects_what_the_fan_cannot_index(built_lib):
    wl = _scene()
    sky = workloads.sky(64, 32)
    with Context(sky, disc=None, emitter=wl.emitter) as ctx:
        p = _params(ctx, wl)
        with pytest.raises(_abi.StError) as e:
            ctx.render_layered_raw(wl.cam, workloads.Kerr(1.0, 0.5), p)
        assert e.value.code == _abi.ST_EUNSUPPORTED
        moving = Camera(wl.cam.pos, wl.cam.fwd, wl.cam.right, wl.cam.up_local, wl.cam.fov_factor,
                        np.array([0.0, 0.1, 0.0]))
        with pytest.raises(_abi.StError) as e:
            ctx.render_layered_raw(moving, wl.bh, p)
        assert e.value.code == _abi.ST_EUNSUPPORTED


def test_fan_cache_follows_the_camera_radius(built_lib):
    wl = _scene(disc=True, w=96, h=54)
    sky = workloads.sky(512, 256)
    other = Camera.look_at((0.0, -25.0, 3.0), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), wl.cam.fov_factor)
    with Context(sky, disc=wl.disc, emitter=wl.emitter) as ctx:
        p = _params(ctx, wl, FP32)
        a = ctx.render_layered_raw(wl.cam, wl.bh, p)
        b = ctx.render_layered_raw(other, wl.bh, p)
        a2 = ctx.render_layered_raw(wl.cam, wl.bh, p)     # fans rebuilt for r = 30
        a3 = ctx.render_layered_raw(wl.cam, wl.bh, p)     # fans reused
        fan_a, _, _ = ctx.sky_fan(wl.cam, wl.bh, p)
        fan_b, _, _ = ctx.sky_fan(other, wl.bh, p)
    assert not np.array_equal(a.image, b.image)
    np.testing.assert_array_equal(a.image, a2.image)
    np.testing.assert_array_equal(a.image, a3.image)
    assert not np.array_equal(fan_a, fan_b)


def _fan_rmin(fan, psi):
    """Fan periapsis at the composite's psi, interpolated as the kernel does."""
    n = fan.shape[0]
    t = psi.astype(np.float32) * np.float32(n - 1) / np.float32(math.pi)
    k0 = np.clip(t.astype(np.int64), 0, n - 2)
    fr = t - k0.astype(np.float32)
    return fan[k0, 3] + fr * (fan[k0 + 1, 3] - fan[k0, 3])


def test_ring_pass(built_lib):
    """The foveated ring pass (render_layered_gpu!'s ring_out / ring_rmin,
    src/metal.jl:3102-3118, 2846-2863) over a half-resolution bulk layer:
    - the screen box only skips rays the pass would have made transparent,
      so the frame is bit-identical with and without it;
    - where the fan periapsis is at or above ring_rmin the ring weight is 0
      and the frame is the half-resolution layered frame bit for bit; where
      it is below 0.8 ring_rmin the weight is 1 and the frame is the
      display-resolution layered frame (to the blend's rounding);
    - in the wound region the ring frame is closer to the full trace than
      the half-resolution frame."""
    wl = _scene(disc=True, w=192, h=108)
    sky = workloads.sky(512, 256)
    R = 6.0
    half = (wl.width // 2, wl.height // 2)
    with Context(sky, disc=wl.disc, emitter=wl.emitter) as ctx:
        p = _params(ctx, wl, FP32)
        ring = ctx.render_layered_raw(wl.cam, wl.bh, p, layer_size=half, ring_rmin=R, diag=True)
        nobox = ctx.render_layered_raw(wl.cam, wl.bh, p, layer_size=half, ring_rmin=R, ring_box=False)
        lo = ctx.render_layered_raw(wl.cam, wl.bh, p, layer_size=half)
        hi = ctx.render_layered_raw(wl.cam, wl.bh, p)
        full = ctx.render_raw(wl.cam, wl.bh, p)
        fan, _, _ = ctx.sky_fan(wl.cam, wl.bh, p)
    assert ring.stats["status"] == _abi.ST_OK
    np.testing.assert_array_equal(ring.image, nobox.image)
    rmin = _fan_rmin(fan, ring.diag["lambda_"])
    outer = rmin > R * 1.001
    inner = rmin < 0.8 * R * 0.999
    assert outer.sum() > 0.2 * outer.size and inner.sum() > 100, (outer.sum(), inner.sum())
    np.testing.assert_array_equal(ring.image[outer], lo.image[outer])
    np.testing.assert_allclose(ring.image[inner], hi.image[inner], rtol=1e-5, atol=1e-7)
    lum = np.maximum(full.image.astype(np.float64).sum(-1), 1e-6)
    e_ring = np.abs(ring.image - full.image).sum(-1)[inner] / lum[inner]
    e_lo = np.abs(lo.image - full.image).sum(-1)[inner] / lum[inner]
    print("ring region: half-res median", np.median(e_lo), "ring median", np.median(e_ring),
          "ms", ring.stats["kernel_ms"], nobox.stats["kernel_ms"], lo.stats["kernel_ms"], hi.stats["kernel_ms"])
    assert np.mean(e_ring) < np.mean(e_lo)


def test_layered_with_gas_matches_full_trace(built_lib):
    """The layer pass with a gas volume (the gate is the gas sphere): emission
    is traced identically inside it, the sky comes from the fan outside."""
    from spacetime_gb300.scene import make_volume
    wl = _scene(disc=True, w=160, h=90)
    vol = make_volume(inner=3.0, outer=20.0, nr=96, nphi=64, nz=16, seed=4)
    sky = workloads.sky(512, 256)
    with Context(sky, disc=wl.disc, volume=vol, emitter=wl.emitter) as ctx:
        p = _params(ctx, wl, FP32)
        lay = ctx.render_layered_raw(wl.cam, wl.bh, p)
        full = ctx.render_raw(wl.cam, wl.bh, p)
    assert lay.stats["gas_samples"] > 0 and lay.stats["status"] == _abi.ST_OK
    lum = np.maximum(full.image.astype(np.float64).sum(-1), 1e-6)
    rel = np.abs(lay.image - full.image).sum(-1) / lum
    print("layered + gas vs trace: median", np.median(rel), "p99", np.percentile(rel, 99),
          "gas samples", lay.stats["gas_samples"], full.stats["gas_samples"])
    assert np.median(rel) <= 1e-4
    assert np.percentile(rel, 99) <= 1e-2
