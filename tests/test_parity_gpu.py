"""CUDA path vs the FP64 oracle on identical seeded inputs (through the C ABI).

Tolerances:
  FP64 vs the oracle's fixed-step twin (same step rule, same kill tests):
    escape direction median <= 1e-9 rad, radiance rel. p99 <= 1e-5
    (the two differ only in rounding: the GPU fuses multiply-adds);
  FP64 vs the oracle's Tsit5 (rtol 1e-10): direction median <= 1e-8 rad;
  FP32_GUARDED vs Tsit5: direction median <= 1e-4 rad, p99 <= 1e-3 rad,
    radiance median <= 1e-3 (the target of the mixed-precision path).
Rays whose classification differs (grazing the shadow edge / photon ring,
chaotic under any rounding) are counted and bounded separately.
"""
import numpy as np
import pytest

from oracle import oracle as O
from spacetime_gb300 import _abi, workloads

from .helpers import compare, gpu_render, oracle_scene

pytestmark = pytest.mark.gpu

FP64, FP32, FP32G = _abi.ST_PREC_FP64, _abi.ST_PREC_FP32, _abi.ST_PREC_FP32_GUARDED


@pytest.fixture(scope="module")
def sky():
    return workloads.sky()


def _check_twin(c, n, mismatch_frac=2e-3):
    assert c["class_mismatch"] <= max(2, mismatch_frac * n), c
    assert c["dir_median"] <= 1e-9, c
    assert c["rad_p99"] <= 1e-5, c


def test_config0_render_fp64_vs_twin_and_tsit5(built_lib, sky):
    w = workloads.config0()
    g = gpu_render(w, sky, FP64)
    assert np.isfinite(g.image).all()
    twin, twin_rays = oracle_scene(w, sky, O.INT_RK4).render()
    c = compare(g.image, g.diag, twin, twin_rays)
    _check_twin(c, c["n"])
    ts, ts_rays = oracle_scene(w, sky, O.INT_TSIT5).render()
    c2 = compare(g.image, g.diag, ts, ts_rays)
    assert c2["dir_median"] <= 1e-8 and c2["rad_median"] <= 1e-6, c2
    assert c2["class_mismatch"] <= 0.002 * c2["n"], c2


def test_config0_draft_fp64_vs_twin(built_lib, sky):
    w = workloads.config0()
    w.semantics = _abi.ST_SEM_DRAFT
    w.emitter = _abi.ST_EMIT_KS_EXACT
    w.params = dict(samples=1, pixel_jitter=0, exit_landing=0)
    g = gpu_render(w, sky, FP64)
    ref, rays = oracle_scene(w, sky, O.INT_RK4).render()
    _check_twin(compare(g.image, g.diag, ref, rays), w.width * w.height)


def test_kerr_thin_disc_fp64_vs_twin(built_lib, sky):
    w = workloads.config1_thin().scaled(240, 135)
    w.params = dict(samples=1, pixel_jitter=0, exit_landing=0)
    g = gpu_render(w, sky, FP64)
    ref, rays = oracle_scene(w, sky, O.INT_RK4).render()
    _check_twin(compare(g.image, g.diag, ref, rays), w.width * w.height)


def test_kerr_volume_fp64_vs_twin(built_lib, sky):
    w = workloads.config1().scaled(160, 90)
    g = gpu_render(w, sky, FP64)
    assert g.stats["gas_samples"] > 0
    ref, rays = oracle_scene(w, sky, O.INT_RK4).render()
    _check_twin(compare(g.image, g.diag, ref, rays), w.width * w.height)


@pytest.mark.parametrize("prec", [FP32G, FP32])
def test_kerr_volume_fp32_vs_tsit5(built_lib, sky, prec):
    w = workloads.config1().scaled(192, 108)
    g = gpu_render(w, sky, prec, r_guard=3.0, crit_band=0.05, renorm_every=64)
    ref, rays = oracle_scene(w, sky, O.INT_TSIT5).render()
    c = compare(g.image, g.diag, ref, rays)
    print(_abi.ST_PREC_FP32_GUARDED == prec and "FP32G" or "FP32", c, g.stats)
    if prec == FP32G:
        assert c["dir_median"] <= 1e-4 and c["dir_p99"] <= 1e-3, c
        assert c["rad_median"] <= 1e-3, c
    assert c["class_mismatch"] <= 0.01 * c["n"], c


def test_persistent_schedule_matches_pixel(built_lib, sky):
    """Same rays, same steps; the two kernels are separate float compilations
    (multiply-add contraction may differ), so radiance agrees to 1e-3 relative
    on all but 1 % of pixels rather than bit for bit."""
    w = workloads.config1().scaled(200, 120)
    a = gpu_render(w, sky, FP32G, schedule=_abi.ST_SCHED_PIXEL)
    b = gpu_render(w, sky, FP32G, schedule=_abi.ST_SCHED_PERSISTENT, chunk_steps=16)
    assert b.stats["status"] == _abi.ST_OK
    assert a.stats["steps"] == b.stats["steps"]
    rel = np.abs(a.image - b.image).sum(-1) / np.maximum(np.abs(a.image).sum(-1), 1e-6)
    assert (rel > 1e-3).mean() <= 0.01, (rel > 1e-3).mean()
    c = compare(b.image, b.diag, a.image.astype(np.float64), a.diag)
    assert c["class_mismatch"] <= 2 and c["dir_median"] <= 1e-5, c


@pytest.mark.parametrize("order,twin", [(45, O.INT_TSIT5_K45), (46, O.INT_TSIT5_K46)])
def test_adaptive_tsit5_modes_fp64_vs_twin(built_lib, sky, order, twin):
    """render_draft_mtl(...; order=45/46): the kernel's adaptive Tsitouras 5(4)
    with FSAL and PI control, against the oracle's restatement of the same
    controller (src/metal.jl:1278-1381)."""
    w = workloads.config1_thin().scaled(160, 90)
    w.params = dict(samples=1, pixel_jitter=0, exit_landing=1)
    g = gpu_render(w, sky, FP64, order=order, tol=1e-6)
    ref, rays = oracle_scene(w, sky, twin, tol=1e-6).render()
    c = compare(g.image, g.diag, ref, rays)
    assert c["class_mismatch"] <= max(2, 2e-3 * c["n"]), c
    assert c["dir_median"] <= 1e-9 and c["rad_p99"] <= 1e-5, c
    # and it is a converged integrator: against the oracle's Tsit5 at rtol 1e-10
    ts, ts_rays = oracle_scene(w, sky, O.INT_TSIT5).render()
    c2 = compare(g.image, g.diag, ts, ts_rays)
    assert c2["dir_median"] <= 1e-6, c2


def test_guarded_deferral_matches_inline_guards(built_lib, sky, monkeypatch):
    """FP32_GUARDED on the pixel schedule with SPACETIME_GB300_GUARD_DEFER=1
    stops each ray before its first FP64 guard step and resumes the saved rays
    one per thread, so their FP64 steps start in full warps.  Against the
    default (guard steps inline): the same rays take the same steps, FP64
    steps included, and the frames agree to the float tolerance of two
    compilations of one kernel (radiance within 1e-3 on 99 % of pixels)."""
    w = workloads.config1().scaled(240, 135)
    kw = dict(r_guard=3.0, crit_band=0.05, crit_r=4.0, renorm_every=256)
    monkeypatch.setenv("SPACETIME_GB300_GUARD_DEFER", "1")
    a = gpu_render(w, sky, FP32G, **kw)
    monkeypatch.delenv("SPACETIME_GB300_GUARD_DEFER")
    b = gpu_render(w, sky, FP32G, **kw)
    print("deferred", a.stats, "inline", b.stats)
    assert a.stats["status"] == _abi.ST_OK and a.stats["rays"] == w.width * w.height
    assert a.stats["fp64_steps"] > 0
    assert abs(a.stats["steps"] - b.stats["steps"]) <= 1e-4 * b.stats["steps"]
    assert abs(a.stats["fp64_steps"] - b.stats["fp64_steps"]) <= 1e-3 * b.stats["fp64_steps"]
    rel = np.abs(a.image - b.image).sum(-1) / np.maximum(np.abs(b.image).sum(-1), 1e-6)
    assert (rel > 1e-3).mean() <= 0.01, (rel > 1e-3).mean()
    c = compare(a.image, a.diag, b.image.astype(np.float64), b.diag)
    assert c["class_mismatch"] <= 2 and c["dir_median"] <= 1e-6, c
    # the diag flags carry no internal bits
    assert not (a.diag["flags"] & ~0x1FF).any()


def test_blackbody_table_in_shared_memory(built_lib, sky, monkeypatch):
    """SPACETIME_GB300_LUT_SMEM=1 stages the blackbody table in each block's
    shared memory before the pixel kernel takes rays; the lookups read the same
    entries, so the frame is bit-identical to the L1 path (gas and thin disc)."""
    for w in (workloads.config1().scaled(160, 90), workloads.config1_thin().scaled(160, 90)):
        a = gpu_render(w, sky, FP32, diag=False)
        monkeypatch.setenv("SPACETIME_GB300_LUT_SMEM", "1")
        b = gpu_render(w, sky, FP32, diag=False)
        monkeypatch.delenv("SPACETIME_GB300_LUT_SMEM")
        np.testing.assert_array_equal(a.image, b.image)
        assert a.stats["steps"] == b.stats["steps"]


def test_double_float_guards_match_fp64_guards(built_lib, sky):
    """ST_PREC_FP32_GUARDED_DF runs the guarded path's guard steps and null
    renormalisation in double-float arithmetic on the FP32 pipe (about 47-bit
    significands) instead of FP64.  Both round each result into the same
    float-float state (about 48 bits), so the guard decisions and the rays'
    steps are the same, and the frames agree far inside the float tolerance:
    exit directions within 1e-9 rad at the median, radiance within 1e-5 on
    99 % of pixels (Kerr with gas, and Schwarzschild with a disc)."""
    kw = dict(r_guard=3.0, crit_band=0.05, crit_r=4.0, renorm_every=256)
    for w in (workloads.config1().scaled(240, 135), workloads.config0()):
        if w.semantics == _abi.ST_SEM_RENDER:
            w = workloads.config0()
            w.semantics, w.emitter = _abi.ST_SEM_DRAFT, _abi.ST_EMIT_KS_EXACT
            w.params = dict(samples=1, pixel_jitter=0, exit_landing=1)
        a = gpu_render(w, sky, FP32G, **kw)
        b = gpu_render(w, sky, _abi.ST_PREC_FP32_GUARDED_DF, **kw)
        print(w.name, a.stats, b.stats)
        assert a.stats["fp64_steps"] > 0 and b.stats["fp64_steps"] > 0
        assert abs(a.stats["steps"] - b.stats["steps"]) <= 1e-5 * a.stats["steps"]
        assert abs(a.stats["fp64_steps"] - b.stats["fp64_steps"]) <= 1e-4 * a.stats["fp64_steps"]
        rel = np.abs(a.image - b.image).sum(-1) / np.maximum(np.abs(a.image).sum(-1), 1e-6)
        assert np.percentile(rel, 99) <= 1e-5, np.percentile(rel, 99)
        c = compare(b.image, b.diag, a.image.astype(np.float64), a.diag)
        assert c["class_mismatch"] <= 2 and c["dir_median"] <= 1e-9, c
