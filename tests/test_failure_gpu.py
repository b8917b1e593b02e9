"""Device-side failure detection, driven from the host with nothing faulted.

- The persistent kernel's outer loop is bounded by an iteration budget; the
  environment variable SPACETIME_GB300_QUEUE_BUDGET lowers it so the queue
  runs out.  The kernel records ST_EBUDGET in the status word and returns;
  the call reports it, and the same context renders correctly afterwards.
- Every mbarrier wait of the tcgen05 network kernel is bounded.
  SPACETIME_GB300_TC_WAIT_OUT=1 leaves each CTA's first copies unissued (a
  barrier nothing completes) with a short bound, so every CTA's first wait
  runs out with nothing in flight.  The kernel leaves all its tiles failed, frees
  its TMEM and returns: st_surrogate_forward_tc reports ST_ECUDA, a surrogate
  frame integrates every pixel (the plain frame, exactly) and reports the
  status, and both work normally on the next call.
"""
import numpy as np
import pytest

from spacetime_gb300 import _abi, workloads
from spacetime_gb300.api import Context

pytestmark = pytest.mark.gpu


def _scene():
    w = workloads.config1_thin().scaled(96, 54)
    w.params = dict(samples=1, pixel_jitter=0, exit_landing=1)
    w.disc = None
    return w


def test_persistent_queue_budget_runs_out(built_lib, monkeypatch):
    w = _scene()
    sky = workloads.sky(512, 256)
    with Context(sky, disc=w.disc, emitter=w.emitter) as ctx:
        p = ctx.params(w.semantics, width=w.width, height=w.height, precision=_abi.ST_PREC_FP32,
                       schedule=_abi.ST_SCHED_PERSISTENT, chunk_steps=16, **w.params)
        pix = ctx.params(w.semantics, width=w.width, height=w.height, precision=_abi.ST_PREC_FP32, **w.params)
        monkeypatch.setenv("SPACETIME_GB300_QUEUE_BUDGET", "3")
        img = np.zeros((w.height, w.width, 3), np.float32)
        with pytest.raises(_abi.StError) as e:
            ctx.render_raw(w.cam, w.bh, p, out=img)
        assert e.value.code == _abi.ST_EBUDGET
        monkeypatch.delenv("SPACETIME_GB300_QUEUE_BUDGET")
        a = ctx.render_raw(w.cam, w.bh, p)
        b = ctx.render_raw(w.cam, w.bh, pix)
    assert a.stats["status"] == _abi.ST_OK and a.stats["rays"] == w.width * w.height
    assert a.stats["steps"] == b.stats["steps"]
    rel = np.abs(a.image - b.image).sum(-1) / np.maximum(np.abs(b.image).sum(-1), 1e-6)
    assert (rel > 1e-3).mean() <= 0.01


def test_tensor_core_wait_runs_out(built_lib, monkeypatch):
    from spacetime_gb300.surrogate import load_trained
    sur = load_trained()
    X, _, _ = sur.generate(300, offset=7, copy=True)
    good = sur.forward_tc(X)
    monkeypatch.setenv("SPACETIME_GB300_TC_WAIT_OUT", "1")
    with pytest.raises(_abi.StError) as e:
        sur.forward_tc(X)
    assert e.value.code == _abi.ST_ECUDA
    w = _scene()
    sky = workloads.sky(512, 256)
    with Context(sky, disc=None, emitter=w.emitter) as ctx:
        ctx.set_surrogate(sur)
        plain = ctx.params(w.semantics, width=w.width, height=w.height, precision=_abi.ST_PREC_FP32, **w.params)
        served = ctx.params(w.semantics, width=w.width, height=w.height, precision=_abi.ST_PREC_FP32, surrogate=1,
                            surrogate_sigma=4e-4, **w.params)
        ref = ctx.render_raw(w.cam, w.bh, plain)
        img = np.zeros((w.height, w.width, 3), np.float32)
        with pytest.raises(_abi.StError) as e:
            ctx.render_raw(w.cam, w.bh, served, out=img)
        assert e.value.code == _abi.ST_ECUDA
        np.testing.assert_array_equal(img, ref.image)   # every tile went to the integrator
        monkeypatch.delenv("SPACETIME_GB300_TC_WAIT_OUT")
        again = ctx.render_raw(w.cam, w.bh, served)
    assert again.stats["status"] == _abi.ST_OK and again.stats["surrogate_rays"] > 0
    np.testing.assert_array_equal(sur.forward_tc(X), good)
    sur.close()
