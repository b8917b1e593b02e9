"""Camera tracks (st_render_frames): one launch for all frames, on either
schedule, with or without CUDA-graph replay, must reproduce the per-frame
renders; frames with the camera inside the horizon must match the oracle's
FP64 twin.

Exactness: the same kernel (one schedule, graph or not, one frame or many)
is bit-exact.  The pixel and persistent kernels are separate FP32 fast-math
compilations whose multiply-add contraction may differ, so across schedules
the bar is relative radiance 1e-3 on all but 1% of pixels."""
import numpy as np
import pytest

from oracle import oracle as O
from spacetime_gb300 import _abi, autotune, workloads
from spacetime_gb300.api import Context
from spacetime_gb300.scene import lens_fov
from spacetime_gb300.ship import free_fall_track

from .helpers import compare, gpu_render, oracle_scene

pytestmark = pytest.mark.gpu

W, H = 96, 54


@pytest.fixture(scope="module")
def track():
    return workloads.config2(nframes=12, width=W, height=H)


@pytest.fixture(scope="module")
def sky():
    return workloads.sky(512, 256)


def _params(ctx, w, **kw):
    return ctx.params(_abi.ST_SEM_DRAFT, width=W, height=H, samples=1, pixel_jitter=0, exit_landing=1,
                      nmax=w.params["nmax"], precision=_abi.ST_PREC_FP32, **kw)


def test_track_schedules_graph_and_single_frames_agree(built_lib, track, sky):
    w = track
    with Context(sky, disc=w.disc, emitter=w.emitter) as ctx:
        a = ctx.render_frames_raw(w.cams, w.bh, _params(ctx, w, schedule=_abi.ST_SCHED_PIXEL))
        b = ctx.render_frames_raw(w.cams, w.bh, _params(ctx, w, schedule=_abi.ST_SCHED_PERSISTENT, chunk_steps=32))
        g1 = ctx.render_frames_raw(w.cams, w.bh, _params(ctx, w, schedule=_abi.ST_SCHED_PERSISTENT, graph=1))
        # replay with a different track: the graph must pick up the new cameras
        cams2 = list(reversed(w.cams))
        g2 = ctx.render_frames_raw(cams2, w.bh, _params(ctx, w, schedule=_abi.ST_SCHED_PERSISTENT, graph=1))
        singles = [ctx.render_raw(c, w.bh, _params(ctx, w)).image for c in w.cams]
    for r in (a, b, g1, g2):
        assert r.stats["status"] == _abi.ST_OK
        assert r.stats["rays"] == len(w.cams) * W * H
    np.testing.assert_array_equal(b.image, g1.image)
    np.testing.assert_array_equal(g2.image, g1.image[::-1])
    np.testing.assert_array_equal(a.image, np.stack(singles))
    rel = np.abs(a.image - b.image).sum(-1) / np.maximum(np.abs(a.image).sum(-1), 1e-6)
    assert (rel > 1e-3).mean() <= 0.01, (rel > 1e-3).mean()


def test_interior_frames_match_twin(built_lib, track, sky):
    """The last frames sit inside the horizon (r < 2M): rays leave through it,
    the floor is 0.3M, the tetrad is the 2.5M free-faller, boosted."""
    w = track
    inside = [c for c in w.cams if np.linalg.norm(c.pos) < 2.0]
    assert inside, "the track ends inside the horizon"
    # two more, released from rest at 3M, at r ~ 1.9M and ~0.7M
    inside += [c for c in free_fall_track(3.0, 0.8, 5, M=1.0, incl_deg=85.0, fov=lens_fov(24.0))[-2:]]
    for cam in inside:
        assert np.linalg.norm(cam.pos) < 2.0
        one = workloads.Workload("interior", w.bh, cam, 48, 27, _abi.ST_SEM_DRAFT, w.disc, w.emitter,
                                 params=dict(samples=1, pixel_jitter=0, exit_landing=1, nmax=20000))
        g = gpu_render(one, sky, _abi.ST_PREC_FP64)
        ref, rays = oracle_scene(one, sky, O.INT_RK4).render()
        c = compare(g.image, g.diag, ref, rays)
        assert np.isfinite(g.image).all()
        assert c["class_mismatch"] <= 2 and c["dir_median"] <= 1e-9 and c["rad_p99"] <= 1e-5, c


def test_autotuner_caches_a_choice(built_lib, track, sky, tmp_path, monkeypatch):
    monkeypatch.setenv("SPACETIME_GB300_AUTOTUNE", str(tmp_path / "tune.json"))
    w = track
    with Context(sky, disc=w.disc, emitter=w.emitter) as ctx:
        p = _params(ctx, w)
        e = autotune.tune(ctx, w.cams, w.bh, p, sample_frames=4, repeats=1)
        assert e["schedule"] in ("pixel", "persistent") and len(e["ms"]) == len(autotune.CANDIDATES)
        again = autotune.tune(ctx, w.cams, w.bh, p)
        assert again == e
        autotune.apply(p, e)
        r = ctx.render_frames_raw(w.cams, w.bh, p)
        assert r.stats["status"] == _abi.ST_OK
