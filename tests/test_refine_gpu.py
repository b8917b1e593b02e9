"""Adaptive refinement (render_draft_mtl `refine`, src/metal.jl:2104-2240) on the
GPU: the base passes record per-ray luminance moments and the Bardeen graze
fraction; the flagged pixels' bounding box (+ margin) is re-rendered refine-1
more times with fresh strata and renormalised.

- Without jitter every pass traces the same ray, so refinement must leave the
  frame unchanged (to float rounding of the renormalisation).
- With jitter, pixels outside the box are the base render bit for bit, the
  changed pixels lie in one box, and the ray count grows by exactly the box's
  area x passes x (refine - 1).
"""
import numpy as np
import pytest

from spacetime_gb300 import _abi, workloads
from spacetime_gb300.api import Context

pytestmark = pytest.mark.gpu


def _scene():
    w = workloads.config4(nframes=1).scaled(128, 72)   # Kerr a=0.99: a wide graze zone
    w.vol = None
    w.params = dict(exit_landing=1)
    return w


def test_refinement_without_jitter_changes_nothing(built_lib):
    w = _scene()
    sky = workloads.sky(512, 256)
    with Context(sky, disc=w.disc, emitter=w.emitter) as ctx:
        kw = dict(width=w.width, height=w.height, precision=_abi.ST_PREC_FP32, samples=1, pixel_jitter=0, **w.params)
        a = ctx.render_raw(w.cam, w.bh, ctx.params(w.semantics, **kw))
        b = ctx.render_raw(w.cam, w.bh, ctx.params(w.semantics, refine=3, **kw))
    assert b.stats["status"] == _abi.ST_OK
    assert b.stats["launches"] == 3, b.stats   # the box was found and refined twice
    np.testing.assert_allclose(b.image, a.image, rtol=2e-6, atol=1e-12)


def test_refinement_box_and_ray_count(built_lib):
    w = _scene()
    sky = workloads.sky(512, 256)
    with Context(sky, disc=w.disc, emitter=w.emitter) as ctx:
        kw = dict(width=w.width, height=w.height, precision=_abi.ST_PREC_FP32, samples=2, pixel_jitter=1, seed=11,
                  **w.params)
        a = ctx.render_raw(w.cam, w.bh, ctx.params(w.semantics, **kw))
        b = ctx.render_raw(w.cam, w.bh, ctx.params(w.semantics, refine=3, refine_margin=4, **kw))
    changed = np.any(a.image != b.image, axis=-1)
    assert changed.any()
    js, is_ = np.nonzero(changed)
    box = (is_.min(), js.min(), is_.max() + 1, js.max() + 1)
    inside = np.zeros_like(changed)
    inside[box[1]:box[3], box[0]:box[2]] = True
    # outside the box: the base render, bit for bit
    np.testing.assert_array_equal(a.image[~inside], b.image[~inside])
    area = (box[2] - box[0]) * (box[3] - box[1])
    extra = b.stats["rays"] - a.stats["rays"]
    # the box found from the changed pixels can be smaller than the refined one
    # (a pixel may come out equal); the refined box's area divides the extra rays
    assert extra % (4 * 2) == 0 and extra // 8 >= area, (extra, area)
    assert b.stats["launches"] == 4 * 3


def test_refinement_is_a_draft_feature(built_lib):
    w = workloads.config0().scaled(32, 18)
    with Context(workloads.sky(64, 32), disc=w.disc, emitter=w.emitter) as ctx:
        with pytest.raises(_abi.StError) as e:
            ctx.render_raw(w.cam, w.bh, ctx.params(w.semantics, width=32, height=18, refine=2))
        assert e.value.code == _abi.ST_EUNSUPPORTED
