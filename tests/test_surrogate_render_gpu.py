"""The surrogate inside st_render (camera-ray mode): gating, compaction of
the integrated remainder, and what a trained network gains.

- An untrained network is never confident, so every ray falls back to the
  integrator and the frame must equal the plain render bit for bit.
- With a trained network (trained here, on the GPU, in seconds) served rays
  skip the integration: the trace kernel's step count drops, and the served
  rays' exit directions stay within the gate's error level against the FP64
  oracle's Tsit5.
"""
import numpy as np
import pytest

from oracle import oracle as O
from spacetime_gb300 import _abi, workloads
from spacetime_gb300.api import Context
from spacetime_gb300.surrogate import Surrogate

from .helpers import angle

pytestmark = pytest.mark.gpu


def _scene(disc=True):
    w = workloads.config1_thin().scaled(192, 108)
    w.params = dict(samples=1, pixel_jitter=0, exit_landing=1)
    if not disc:
        w.disc = None
    return w


def test_untrained_surrogate_falls_back_everywhere(built_lib):
    w = _scene()
    sky = workloads.sky(512, 256)
    sur = Surrogate(0, seed=9)
    with Context(sky, disc=w.disc, emitter=w.emitter) as ctx:
        ctx.set_surrogate(sur)
        p0 = ctx.params(w.semantics, width=w.width, height=w.height, precision=_abi.ST_PREC_FP32, **w.params)
        a = ctx.render_raw(w.cam, w.bh, p0, diag=True)
        p1 = ctx.params(w.semantics, width=w.width, height=w.height, precision=_abi.ST_PREC_FP32, surrogate=1,
                        surrogate_sigma=1e-4, **w.params)
        b = ctx.render_raw(w.cam, w.bh, p1, diag=True)
    assert b.stats["surrogate_rays"] == 0
    np.testing.assert_array_equal(a.image, b.image)
    assert a.stats["steps"] == b.stats["steps"]
    sur.close()


def test_trained_surrogate_gain(built_lib):
    """Config1's camera and hole with no disc: every ray either escapes or
    falls in, so the gate is set by the network's confidence alone."""
    w = _scene(disc=False)
    sky = workloads.sky(512, 256)
    sur = Surrogate(0, seed=1)
    sur.generate(1 << 21, offset=0, copy=False)
    for k in range(12):
        lr = 1e-5 + 0.5 * (2e-3 - 1e-5) * (1 + np.cos(np.pi * k / 11))
        sur.train(2000, batch=16384, lr=lr, weight_decay=1e-6)
    with Context(sky, disc=None, emitter=w.emitter) as ctx:
        ctx.set_surrogate(sur)
        p0 = ctx.params(w.semantics, width=w.width, height=w.height, precision=_abi.ST_PREC_FP32, **w.params)
        a = ctx.render_raw(w.cam, w.bh, p0, diag=True)
        p1 = ctx.params(w.semantics, width=w.width, height=w.height, precision=_abi.ST_PREC_FP32, surrogate=1,
                        surrogate_sigma=1e-3, **w.params)
        b = ctx.render_raw(w.cam, w.bh, p1, diag=True)
    served = (b.diag["flags"] & _abi.ST_RAY_SURROGATE) > 0
    print("served fraction", served.mean(), "steps", a.stats["steps"], "->", b.stats["steps"],
          "kernel ms", a.stats["kernel_ms"], "->", b.stats["kernel_ms"])
    assert served.mean() > 0.2
    assert b.stats["steps"] < (1.0 - 0.5 * served.mean()) * a.stats["steps"]
    assert b.stats["surrogate_rays"] == served.sum()
    assert np.isfinite(b.image).all()
    ref, rays = O.scene_for(w, sky, O.INT_TSIT5).render()
    ok = served & ((rays["flags"] & O.RAY_ESCAPED) > 0)
    d = angle(b.diag["dir"][ok], rays["dir"][ok])
    print("served dir error median", np.median(d), "p99", np.percentile(d, 99))
    assert np.median(d) < 1e-3
    # unserved pixels are the integrator's, bit for bit
    np.testing.assert_array_equal(a.image[~served], b.image[~served])
    sur.close()


def test_tcgen05_frame_kernel_matches_mma_sync(built_lib, monkeypatch):
    """The frame pass on tcgen05 / TMEM and on mma.sync computes the same
    network on the same inputs: the same pixels are served, with the same
    exit directions up to bf16 rounding.  The two kernels reach each
    pre-activation to FP32 accuracy by different summations (layer 0: an FP32
    FMA chain on mma.sync, a split-bf16 product on tcgen05), so a unit whose
    value sits on a bf16 rounding boundary can round the other way, one bf16
    ulp; a ray with such a unit upstream moves by up to ~1e-3 rad.  Measured
    on a GB300: median 2.2e-7 rad, p99 4.3e-4, max 1.6e-3."""
    from spacetime_gb300.surrogate import load_trained
    w = _scene(disc=False)
    sky = workloads.sky(512, 256)
    sur = load_trained()
    out = {}
    with Context(sky, disc=None, emitter=w.emitter) as ctx:
        ctx.set_surrogate(sur)
        p = ctx.params(w.semantics, width=w.width, height=w.height, precision=_abi.ST_PREC_FP32, surrogate=1,
                       surrogate_sigma=4e-4, **w.params)
        for mode in ("sync", "tc"):
            monkeypatch.setenv("SPACETIME_GB300_SURROGATE_MMA", mode)
            out[mode] = ctx.render_raw(w.cam, w.bh, p, diag=True)
    a, b = out["sync"], out["tc"]
    assert a.stats["status"] == _abi.ST_OK and b.stats["status"] == _abi.ST_OK
    sa = (a.diag["flags"] & _abi.ST_RAY_SURROGATE) > 0
    sb = (b.diag["flags"] & _abi.ST_RAY_SURROGATE) > 0
    print("served", sa.mean(), sb.mean(), "disagree", (sa != sb).mean())
    assert sa.mean() > 0.2
    assert (sa != sb).mean() <= 0.005
    both = sa & sb
    d = angle(a.diag["dir"][both], b.diag["dir"][both])
    print("direction difference median", np.median(d), "p99", np.percentile(d, 99), "max", d.max(),
          "fraction above 1e-5", (d > 1e-5).mean())
    assert np.median(d) <= 1e-6 and np.percentile(d, 99) <= 1e-3 and d.max() <= 1e-2
    sur.close()


def test_surrogate_on_a_camera_track(built_lib):
    """st_render_frames with the surrogate: a short track of static cameras
    (config 1's hole, cameras at r = 14-16 M, inclination 80 deg, stepped in
    azimuth; no disc, no gas) runs frame by frame through the single-frame
    path, so each frame equals st_render of its camera bit for bit, rays are
    served, and the stats are the frames' sums.  A track with one camera
    inside r = 4 M (outside the network's domain) is refused whole, and so is
    a context with gas, as st_render refuses it."""
    from spacetime_gb300.scene import Camera, kerr_position, lens_fov
    from spacetime_gb300.surrogate import load_trained
    w = _scene(disc=False)
    sky = workloads.sky(512, 256)
    sur = load_trained()

    def cam(r, phi):
        x, y, z = kerr_position(r, 80.0, 0.9)
        c, s = np.cos(phi), np.sin(phi)
        return Camera.look_at((c * x - s * y, s * x + c * y, z), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), lens_fov(24.0))

    cams = [cam(15.0, 0.0), cam(16.0, 0.4), cam(14.0, 0.8)]
    with Context(sky, disc=None, emitter=w.emitter) as ctx:
        ctx.set_surrogate(sur)
        p = ctx.params(w.semantics, width=w.width, height=w.height, precision=_abi.ST_PREC_FP32, surrogate=1,
                       surrogate_sigma=4e-4, **w.params)
        track = ctx.render_frames_raw(cams, w.bh, p)
        singles = [ctx.render_raw(c, w.bh, p) for c in cams]
        with pytest.raises(_abi.StError) as e:
            ctx.render_frames_raw(cams[:2] + [cam(3.0, 0.0)], w.bh, p)
        assert e.value.code == _abi.ST_EUNSUPPORTED
    assert track.stats["status"] == _abi.ST_OK
    for f, one in enumerate(singles):
        np.testing.assert_array_equal(track.image[f], one.image)
    for key in ("rays", "steps", "surrogate_rays", "launches"):
        assert track.stats[key] == sum(one.stats[key] for one in singles), key
    assert track.stats["surrogate_rays"] > 0.2 * len(cams) * w.width * w.height
    wg = workloads.config1().scaled(w.width, w.height)
    with Context(sky, disc=wg.disc, volume=wg.vol, emitter=wg.emitter) as ctx:
        ctx.set_surrogate(sur)
        p = ctx.params(wg.semantics, width=w.width, height=w.height, precision=_abi.ST_PREC_FP32, surrogate=1,
                       surrogate_sigma=4e-4, **w.params)
        with pytest.raises(_abi.StError) as e:
            ctx.render_frames_raw(cams, wg.bh, p)
        assert e.value.code == _abi.ST_EUNSUPPORTED
    sur.close()
