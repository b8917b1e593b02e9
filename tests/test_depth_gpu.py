"""Depth buckets on the GPU (st_render_depth = render_depth_mtl,
src/metal.jl:1935-1990) against the oracle's bucketed trace.

Tolerances:
  FP64 vs the oracle's fixed-step twin, bucket for bucket: per-pixel L1 error
    over all 3 nb channels relative to the pixel's total, median <= 1e-6 and
    p99 <= 1e-5.  The buckets are float32 on both sides, as the reference's
    output array is, but the GPU adds each step's emission into them as it
    goes (hundreds of float additions along a ray through the gas) while the
    oracle sums in double and rounds once, so the float accumulation sets
    the scale.  A pixel whose path length sits on a bucket edge to rounding
    moves its emission one bucket over, so pixels above 1e-4 are bounded like
    the plain parity tests' class mismatches (2e-3 of the frame);
  FP32, any size: the buckets summed equal the plain render of the same
    passes (same steps; only the grouping of the float sums differs: one
    bucket takes hundreds of per-step additions along a ray through the
    gas): relative 1e-4 at the 99.99th percentile, 1e-3 at most.
"""
import numpy as np
import pytest

from oracle import oracle as O
from spacetime_gb300 import _abi, workloads
from spacetime_gb300.api import Context, render_depth

from .helpers import oracle_scene

pytestmark = pytest.mark.gpu

NB = 10


@pytest.fixture(scope="module")
def sky():
    return workloads.sky()


def _scene(case):
    if case == "schw_disc":
        w = workloads.config0().scaled(96, 54)
        w.semantics = _abi.ST_SEM_DRAFT
        w.emitter = _abi.ST_EMIT_KS_EXACT
        w.params = dict(samples=1, pixel_jitter=0, exit_landing=0)
    else:
        w = workloads.config1().scaled(96, 54)
    return w


def _depth(ctx, w, precision, nb=NB, **kw):
    params = dict(w.params)
    params.update(kw)
    p = ctx.params(w.semantics, width=w.width, height=w.height, precision=precision, **params)
    return ctx.render_depth_raw(w.cam, w.bh, p, nb)


@pytest.mark.parametrize("case", ["schw_disc", "kerr_gas"])
def test_depth_fp64_vs_twin(built_lib, sky, case):
    w = _scene(case)
    with Context(sky, disc=w.disc, volume=w.vol, emitter=w.emitter) as ctx:
        g = _depth(ctx, w, _abi.ST_PREC_FP64)
    ref = oracle_scene(w, sky, O.INT_RK4).render_depth(NB)
    assert g.image.shape == ref.shape
    gi = g.image.astype(np.float64)
    ri = ref.astype(np.float64)
    tot = np.maximum(ri.sum(axis=(2, 3)), 1e-6)
    rel = np.abs(gi - ri).sum(axis=(2, 3)) / tot
    n = w.width * w.height
    emis = ri[:, :, :-1, :].sum()
    print(case, "median", np.median(rel), "p99", np.percentile(rel, 99), "over 1e-4", int((rel > 1e-4).sum()),
          "emission share", emis / ri.sum())
    assert emis > 0.01 * ri.sum()
    assert np.median(rel) <= 1e-6 and np.percentile(rel, 99) <= 1e-5
    assert (rel > 1e-4).sum() <= max(2, 2e-3 * n)


def test_depth_fp32_sums_to_the_plain_frame(built_lib, sky):
    w = workloads.config1().scaled(960, 540)
    w.params = dict(samples=2, pixel_jitter=1, seed=5, exit_landing=0)
    with Context(sky, disc=w.disc, volume=w.vol, emitter=w.emitter) as ctx:
        d = _depth(ctx, w, _abi.ST_PREC_FP32)
        p = ctx.params(w.semantics, width=w.width, height=w.height, precision=_abi.ST_PREC_FP32, **w.params)
        plain = ctx.render_raw(w.cam, w.bh, p)
    assert d.stats["rays"] == plain.stats["rays"] and d.stats["steps"] == plain.stats["steps"]
    s = d.image.astype(np.float64).sum(axis=2)
    rel = np.abs(s - plain.image) / np.maximum(np.abs(plain.image), 1e-3)
    print("buckets summed vs plain: p99.99", np.percentile(rel, 99.99), "max", rel.max())
    assert np.percentile(rel, 99.99) <= 1e-4 and rel.max() <= 1e-3
    # gas emission spreads over several path lengths
    per_bucket = d.image[:, :, :-1, :].sum(axis=(0, 1, 3))
    assert (per_bucket > 1e-3 * per_bucket.sum()).sum() >= 3, per_bucket


def test_depth_sky_only_and_errors(built_lib, sky):
    w = workloads.config0().scaled(64, 36)
    with Context(sky) as ctx:
        img = render_depth(ctx, w.cam, w.bh, width=64, height=36, samples=1, nbuckets=3, precision="fp32")
        assert img.shape == (36, 64, 3, 3)
        assert np.all(img[:, :, :2, :] == 0.0) and img[:, :, 2, :].max() > 0.0
        with pytest.raises(ValueError):
            render_depth(ctx, w.cam, w.bh, width=64, height=36, nbuckets=2)
        p = ctx.params(_abi.ST_SEM_DRAFT, width=64, height=36)
        with pytest.raises(_abi.StError) as e:
            ctx.render_depth_raw(w.cam, w.bh, p, 2)
        assert e.value.code == _abi.ST_EINVAL
        p = ctx.params(_abi.ST_SEM_RENDER, width=64, height=36)
        with pytest.raises(_abi.StError) as e:
            ctx.render_depth_raw(w.cam, w.bh, p, 4)
        assert e.value.code == _abi.ST_EUNSUPPORTED
