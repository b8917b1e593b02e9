"""Projections, thin-lens depth of field, jittered passes and adaptive
refinement on the GPU against the oracle (render_draft_mtl's camera block and
pass loop, src/metal.jl:863-949, 2091-2240).

Each GPU render here is FP64 through the C ABI; the oracle renders the same
passes with its fixed-step FP64 twin (same step rule and kill tests), the
strata of every pass taken from a restatement of the host's pass plan
(tests/helpers.py pass_plan).  Tolerances are the FP64-vs-twin ones of
tests/test_parity_gpu.py: exit direction median <= 1e-9 rad, radiance p99
<= 1e-5, at most 0.2 % of rays (near the shadow edge) classified differently.
"""
import numpy as np
import pytest

from oracle import oracle as O
from spacetime_gb300 import _abi, workloads
from spacetime_gb300.api import Context

from .helpers import compare, oracle_pass, oracle_scene, pass_plan

pytestmark = pytest.mark.gpu

FP64, FP32 = _abi.ST_PREC_FP64, _abi.ST_PREC_FP32


def _check_twin(c, n):
    assert c["class_mismatch"] <= max(2, 2e-3 * n), c
    assert c["dir_median"] <= 1e-9, c
    assert c["rad_p99"] <= 1e-5, c


def _thin(width=160, height=90):
    w = workloads.config1_thin().scaled(width, height)
    w.params = dict(samples=1, pixel_jitter=0, exit_landing=1)
    return w


def _render(w, sky, prec, diag=True, **kw):
    with Context(sky, disc=w.disc, volume=w.vol, emitter=w.emitter) as ctx:
        params = dict(w.params)
        params.update(kw)
        p = ctx.params(w.semantics, width=w.width, height=w.height, precision=prec, **params)
        return ctx.render_raw(w.cam, w.bh, p, diag=diag)


def _oracle_passes(w, sky, plan, aperture_radius=0.0, integrator=O.INT_RK4):
    """The oracle's average of the planned passes (equal weights, as the
    kernel accumulates them) and the last pass's per-ray records."""
    acc, rays = None, None
    for pp in plan:
        sc = oracle_pass(oracle_scene(w, sky, integrator), pp, aperture_radius)
        img, rays = sc.render()
        acc = img.astype(np.float64) if acc is None else acc + img
    return acc / len(plan), rays


@pytest.mark.parametrize("deg", [60.0, 130.0])
def test_fisheye_fp64_vs_twin(built_lib, deg):
    """Equidistant fisheye, half-angle `deg` at the top edge; at 130 deg the
    corners look behind the camera."""
    sky = workloads.sky(512, 256)
    w = _thin()
    w.cam.projection = _abi.ST_PROJ_FISHEYE
    w.cam.fisheye_deg = deg
    g = _render(w, sky, FP64)
    ref, rays = oracle_scene(w, sky, O.INT_RK4).render()
    c = compare(g.image, g.diag, ref, rays)
    print(deg, c)
    assert c["both_escaped"] > 0.2 * c["n"]
    _check_twin(c, c["n"])


def test_fisheye_fp32_vs_tsit5(built_lib):
    sky = workloads.sky(512, 256)
    w = _thin()
    w.cam.projection = _abi.ST_PROJ_FISHEYE
    w.cam.fisheye_deg = 100.0
    g = _render(w, sky, FP32)
    ref, rays = oracle_scene(w, sky, O.INT_TSIT5).render()
    c = compare(g.image, g.diag, ref, rays)
    print(c)
    assert c["dir_median"] <= 1e-4 and c["dir_p99"] <= 1e-3, c
    assert c["rad_median"] <= 1e-3 and c["class_mismatch"] <= 0.005 * c["n"], c


def test_thin_lens_single_pass_fp64_vs_twin(built_lib):
    """Thin lens (aperture 0.8 M, focus on the hole): one pass, one lens
    stratum covering the whole aperture disk, the lens point hashed per pixel."""
    sky = workloads.sky(512, 256)
    w = _thin()
    w.cam.aperture_world = 0.8
    w.cam.focus_dist = 15.0
    g = _render(w, sky, FP64)
    plan = pass_plan(1, 0, 0, w.semantics, dof=True)
    ref, rays = _oracle_passes(w, sky, plan, aperture_radius=0.4)
    c = compare(g.image, g.diag, ref, rays)
    print(c)
    _check_twin(c, c["n"])
    # the lens moved the rays: the pinhole frame differs
    w.cam.aperture_world = 0.0
    pin = _render(w, sky, FP64, diag=False)
    assert np.abs(pin.image - g.image).max() > 1e-3


def test_thin_lens_stratified_passes_fp64_vs_twin(built_lib):
    """samples = 2: four passes, each with its own shuffled lens stratum and
    pixel-jitter stratum; the frame is their average."""
    sky = workloads.sky(512, 256)
    w = _thin(128, 72)
    w.cam.aperture_world = 0.8
    w.cam.focus_dist = 15.0
    g = _render(w, sky, FP64, samples=2, pixel_jitter=1, seed=17)
    assert g.stats["launches"] == 4
    plan = pass_plan(2, 17, 1, w.semantics, dof=True)
    ref, rays = _oracle_passes(w, sky, plan, aperture_radius=0.4)
    c = compare(g.image, g.diag, ref, rays)   # diag: the last pass on both sides
    print(c)
    _check_twin(c, c["n"])


def test_refinement_box_from_the_oracle_moments(built_lib):
    """Adaptive refinement (refine = 2): the oracle renders the four base
    passes, forms each pixel's luminance mean and variance and Bardeen graze
    fraction, flags the pixels whose per-ray std-dev exceeds
    refine_var (E[L] + 0.01) or whose graze fraction exceeds refine_graze
    (src/metal.jl:2189-2240), and widens their bounding box by the margin.
    The GPU's refined box must be that box: the pixels it changed lie inside
    it and span it, and it traced exactly box area x 4 more rays."""
    sky = workloads.sky(512, 256)
    w = workloads.config4(nframes=1).scaled(128, 72)   # Kerr a=0.99, boosted: a wide graze zone
    w.vol = None
    w.params = dict(exit_landing=1)
    S, seed, var, graze, margin = 2, 23, 0.35, 0.05, 8
    kw = dict(samples=S, pixel_jitter=1, seed=seed)
    base = _render(w, sky, FP64, diag=False, **kw)
    ref = _render(w, sky, FP64, diag=False, refine=2, refine_var=var, refine_graze=graze, refine_margin=margin,
                  **kw)
    plan = pass_plan(S, seed, 1, w.semantics, dof=False)
    L, L2, gz = 0.0, 0.0, 0.0
    acc = 0.0
    for pp in plan:
        img, rays = oracle_pass(oracle_scene(w, sky, O.INT_RK4), pp).render()
        lum = 0.2126 * img[..., 0] + 0.7152 * img[..., 1] + 0.0722 * img[..., 2]
        L = L + lum / len(plan)
        L2 = L2 + lum * lum / len(plan)
        gz = gz + ((rays["flags"] & O.RAY_GRAZE) > 0) / len(plan)
        acc = acc + img.astype(np.float64) / len(plan)
    # the base passes themselves match the twin
    rel = np.abs(base.image - acc).sum(-1) / np.maximum(acc.sum(-1), 1e-6)
    assert np.percentile(rel, 99) <= 1e-5
    s2 = L2 - L * L
    flag = ((s2 > 0) & (np.sqrt(np.maximum(s2, 0)) > var * (L + 0.01))) | (gz > graze)
    assert flag.any() and not flag.all()
    rows, cols = np.nonzero(flag)
    Hh, Ww = flag.shape
    c0, r0 = max(cols.min() - margin, 0), max(rows.min() - margin, 0)
    c1, r1 = min(cols.max() + 1 + margin, Ww), min(rows.max() + 1 + margin, Hh)
    area = (c1 - c0) * (r1 - r0)
    print("oracle box", (c0, c1, r0, r1), "flagged", int(flag.sum()), "rays", ref.stats["rays"])
    assert ref.stats["rays"] == S * S * (Ww * Hh + area)
    changed = np.any(ref.image != base.image, axis=-1)
    cr, cc = np.nonzero(changed)
    assert cc.min() >= c0 and cc.max() < c1 and cr.min() >= r0 and cr.max() < r1
    # fresh strata change (almost) every pixel of the box: its edges are reached
    assert cc.min() <= c0 + 1 and cc.max() >= c1 - 2 and cr.min() <= r0 + 1 and cr.max() >= r1 - 2
