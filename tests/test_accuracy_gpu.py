"""Accuracy of the benchmarked paths on the benchmarked frame.

The GPU renders config 1 at its full 1920x1080 size (Kerr a=0.9, camera at
r=15 M, i=80 deg, gas 256x64x32, kernel rules, exit landing); the FP64 oracle
renders crops of that same frame: the central 240x135 (shadow, photon ring,
the densest gas) and a 3x3 grid of 80x45 tiles spread over the frame (mostly
escaping rays, so the direction statistics see the whole field).

Targets, FP32 and FP32 + guards (FP64, or double-float on the FP32 pipe),
against the oracle's Tsit5 (rtol 1e-10):
  exit direction median <= 1e-4 rad, p99 <= 1e-3 rad, over rays both sides
  call escaped; radiance relative error (L1 over RGB / oracle L1) median
  <= 1e-3; no more than 0.5 % of rays classified differently.
Radiance p99 <= 2e-3, against Tsit5 and against the oracle's fixed-step FP64
  twin (the same RK4 step schedule as the kernel).  Measured on a GB300: 9.7e-4
  for FP32 and 9.6e-4 for FP32 + guards, against either oracle integrator --
  the tail is the float gas march (sample positions and the blackbody lookup
  in single precision), which both float paths share; exit directions agree
  to 4.4e-7 (FP32) and 5.3e-8 (guarded) rad at the median.

The learned surrogate (shipped network, tcgen05 frame pass) on the same
camera and hole without disc or gas, at the widest gate that keeps the frame
inside the direction target (predicted std-dev 2e-4 rad): the frame's exit
directions (served and integrated rays) median <= 1e-4, p99 <= 1e-3 rad; the
served rays alone p99 <= 1e-3 rad and median <= 3e-4 rad.  The served rays'
median does not reach 1e-4 (measured 2.1e-4, radiance median 2.4 %): with
bf16 hidden activations the network's exit angles carry errors of ~1e-4 rad,
and its predicted std-dev under-states them by about 2x, so no gate serves
rays at the 1e-4 target (at 1e-4 it serves none).
"""
import numpy as np
import pytest

from oracle import mlp_oracle as MO
from oracle import oracle as O
from spacetime_gb300 import _abi, workloads

from .helpers import angle, compare, gpu_render, oracle_scene

pytestmark = pytest.mark.gpu

FP32, FP32G, FP32GDF = _abi.ST_PREC_FP32, _abi.ST_PREC_FP32_GUARDED, _abi.ST_PREC_FP32_GUARDED_DF
GUARDS = dict(r_guard=3.0, crit_band=0.05, crit_r=4.0, renorm_every=256)
W, H = 1920, 1080
# (col0, cols, row0, rows): the central 240x135 and nine 80x45 tiles
CROPS = [((W - 240) // 2, 240, (H - 135) // 2, 135)] + [
    (c, 80, r, 45) for c in (160, 920, 1680) for r in (90, 517, 945)]
# the surrogate's gate (predicted std-dev of the exit angles, rad): the widest
# that keeps the frame inside the direction target; bench.py reports the
# served-ray histogram at this gate and at 4e-4
SERVED_SIGMA = 2e-4


@pytest.fixture(scope="module")
def sky():
    return workloads.sky()


def _crops(img, diag):
    gi = [img[r0:r0 + rh, c0:c0 + cw].reshape(-1, 1, 3) for c0, cw, r0, rh in CROPS]
    gd = [diag[r0:r0 + rh, c0:c0 + cw].reshape(-1, 1) for c0, cw, r0, rh in CROPS]
    return np.concatenate(gi), np.concatenate(gd)


def _oracle_crops(w, sky, integrator):
    imgs, rays = [], []
    for rect in CROPS:
        im, ry = oracle_scene(w, sky, integrator, rect=rect).render()
        imgs.append(im.reshape(-1, 1, 3))
        rays.append(ry.reshape(-1, 1))
    return np.concatenate(imgs), np.concatenate(rays)


@pytest.fixture(scope="module")
def oracle_config1(sky):
    w = workloads.config1()
    return {"tsit5": _oracle_crops(w, sky, O.INT_TSIT5), "twin": _oracle_crops(w, sky, O.INT_RK4)}


@pytest.mark.parametrize("prec", [FP32, FP32G, FP32GDF], ids=["fp32", "fp32_guarded", "fp32_guarded_df"])
def test_config1_1080p_against_the_oracle(built_lib, sky, oracle_config1, prec):
    w = workloads.config1()
    kw = GUARDS if prec in (FP32G, FP32GDF) else {}
    g = gpu_render(w, sky, prec, **kw)
    assert g.image.shape == (H, W, 3) and np.isfinite(g.image).all()
    gi, gd = _crops(g.image, g.diag)
    ts = compare(gi, gd, *oracle_config1["tsit5"])
    tw = compare(gi, gd, *oracle_config1["twin"])
    print("vs Tsit5", ts)
    print("vs FP64 twin", tw)
    n = ts["n"]
    assert ts["both_escaped"] > 0.4 * n, ts       # the statistics cover the field
    assert ts["dir_median"] <= 1e-4 and ts["dir_p99"] <= 1e-3, ts
    assert ts["rad_median"] <= 1e-3 and ts["rad_p99"] <= 2e-3, ts
    assert ts["class_mismatch"] <= 0.005 * n, ts
    assert tw["rad_p99"] <= 2e-3 and tw["dir_p99"] <= 1e-3, tw


def test_surrogate_served_rays_on_the_1080p_frame(built_lib, sky):
    """The frame, and the served rays alone (the rays the gate hands to the
    network, no integration), against the oracle's Tsit5 on crops of the
    full-size frame."""
    from spacetime_gb300.api import Context
    from spacetime_gb300.surrogate import load_trained
    w = workloads.config1_nogas()
    sur = load_trained()
    with Context(sky, disc=None, emitter=w.emitter) as ctx:
        ctx.set_surrogate(sur)
        p = ctx.params(w.semantics, width=W, height=H, precision=FP32, surrogate=1, surrogate_sigma=SERVED_SIGMA,
                       **w.params)
        g = ctx.render_raw(w.cam, w.bh, p, diag=True)
    sur.close()
    assert g.stats["status"] == _abi.ST_OK
    gi, gd = _crops(g.image, g.diag)
    ref, rays = _oracle_crops(w, sky, O.INT_TSIT5)
    served = ((gd["flags"] & _abi.ST_RAY_SURROGATE) > 0)[:, 0]
    esc = ((rays["flags"] & O.RAY_ESCAPED) > 0)[:, 0]
    frac = g.stats["surrogate_rays"] / (W * H)
    assert frac > 0.05 and served.sum() > 1000, (frac, served.sum())
    d = angle(gd["dir"][:, 0][served & esc].astype(np.float64), rays["dir"][:, 0][served & esc])
    rel = (np.abs(gi[:, 0].astype(np.float64) - ref[:, 0]).sum(-1) / np.maximum(ref[:, 0].sum(-1), 1e-6))[served]
    print(f"served {frac:.3f} of the frame; in the crops {served.sum()} rays, {(served & ~esc).sum()} of them "
          f"captured in the oracle; direction median {np.median(d):.3e} p99 {np.percentile(d, 99):.3e} "
          f"max {d.max():.3e}; radiance median {np.median(rel):.3e} p99 {np.percentile(rel, 99):.3e}")
    assert (served & ~esc).sum() <= 0.001 * served.sum()   # the gate serves no captured ray
    assert np.percentile(d, 99) <= 1e-3 and np.median(d) <= 3e-4
    c = compare(gi, gd, ref, rays)   # the whole frame: served and integrated rays
    print("frame", c)
    assert c["dir_median"] <= 1e-4 and c["dir_p99"] <= 1e-3 and c["class_mismatch"] == 0, c


def test_tcgen05_forward_against_the_mlp_oracle(built_lib):
    """The frame pass's tcgen05 / TMEM network kernel on the shipped weights
    and on a freshly initialised network, against the FP64 MLP oracle under
    the same bf16 contract (hidden weights and activations rounded to bf16;
    the kernel carries the FP32 edge layers as split-bf16 products, ~2^-16
    relative): per output, median error <= 1e-4, 99.9th percentile <= 5e-3
    and max <= 1e-2 of that output's scale.  The tail is an activation whose
    value sits on a bf16 rounding boundary and rounds the other way under a
    different FP32 summation order: one bf16 ulp (2^-8 relative) in one unit.
    Measured on a GB300: shipped median 2.5e-8, max 3.8e-3; initialised
    median 6.7e-7, max 6.1e-3.  Against the plain FP64 network (no bf16
    rounding) the error is the contract's own, <= 2e-2 of the largest output
    as in tests/test_surrogate_gpu.py, and against the mma.sync forward (same
    contract, another summation order) the same percentile and max bounds."""
    from spacetime_gb300.surrogate import Surrogate, load_trained
    rng = np.random.default_rng(5)
    for which in ("shipped", "init"):
        sur = load_trained() if which == "shipped" else Surrogate(0, seed=21)
        X, _, _ = sur.generate(1000, offset=12345, copy=True)   # the network's own input distribution
        X = np.concatenate([X, rng.uniform(-1, 1, (300, 6)).astype(np.float32)])   # 1300 rows: a ragged last tile
        P = sur.get_params()
        tc = sur.forward_tc(X).astype(np.float64)
        sync = sur.forward(X).astype(np.float64)
        ref16 = MO.forward_bf16(P, X)
        ref64, _, _ = MO.forward(P, X)
        sur.close()
        cols = [0, 1, 3, 4, 5]          # output 2 is unused
        scale = np.abs(ref16[:, cols]).max(0)
        e16 = np.abs(tc - ref16)[:, cols] / scale
        e64 = np.abs(tc - ref64)[:, cols] / np.abs(ref64[:, cols]).max()
        es = np.abs(tc - sync)[:, cols] / scale
        print(which, "vs bf16 oracle median", np.median(e16), "max", e16.max(), "| vs FP64 max", e64.max(),
              "| vs mma.sync max", es.max())
        assert np.median(e16) <= 1e-4 and np.percentile(e16, 99.9) <= 5e-3 and e16.max() <= 1e-2
        assert e64.max() <= 2e-2
        assert np.percentile(es, 99.9) <= 5e-3 and es.max() <= 1e-2
