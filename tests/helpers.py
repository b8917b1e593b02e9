"""Shared parity machinery: run the CUDA path and the oracle on identical
seeded inputs and compare per ray."""
from __future__ import annotations

import numpy as np

from oracle import oracle as O
from spacetime_gb300 import _abi
from spacetime_gb300.api import Context


def angle(a, b):
    """Angle between unit vectors, accurate near zero."""
    return 2.0 * np.arcsin(np.clip(np.linalg.norm(a - b, axis=-1) / 2.0, 0.0, 1.0))


def oracle_scene(w, sky, integrator, width=None, height=None, rect=None, **kw):
    return O.scene_for(w, sky, integrator, width=width, height=height, rect=rect, **kw)


def gpu_render(w, sky, precision, width=None, height=None, diag=True, ctx=None, **kw):
    own = ctx is None
    if own:
        ctx = Context(sky, disc=w.disc, volume=w.vol, emitter=w.emitter)
    try:
        params = dict(w.params)
        params.update(kw)
        p = ctx.params(w.semantics, width=width or w.width, height=height or w.height,
                       precision=precision, **params)
        return ctx.render_raw(w.cam, w.bh, p, diag=diag)
    finally:
        if own:
            ctx.close()


def compare(gpu_img, gpu_diag, ref_img, ref_rays):
    """Per-ray exit-direction and radiance errors over rays both sides agree escaped."""
    g_esc = (gpu_diag["flags"] & _abi.ST_RAY_ESCAPED) > 0
    o_esc = (ref_rays["flags"] & O.RAY_ESCAPED) > 0
    g_black = (gpu_diag["flags"] & _abi.ST_RAY_BLACK) > 0
    o_black = (ref_rays["flags"] & O.RAY_BLACK) > 0
    both = g_esc & o_esc
    d = angle(gpu_diag["dir"][both].astype(np.float64), ref_rays["dir"][both])
    lum_g = gpu_img.astype(np.float64).sum(-1)
    lum_o = ref_img.astype(np.float64).sum(-1)
    rel = np.abs(gpu_img.astype(np.float64) - ref_img).sum(-1) / np.maximum(lum_o, 1e-6)
    out = dict(
        n=int(gpu_img.shape[0] * gpu_img.shape[1]),
        both_escaped=int(both.sum()),
        class_mismatch=int((g_black != o_black).sum()),
        dir_median=float(np.median(d)) if d.size else 0.0,
        dir_p99=float(np.percentile(d, 99)) if d.size else 0.0,
        dir_max=float(d.max()) if d.size else 0.0,
        rad_median=float(np.median(rel)),
        rad_p99=float(np.percentile(rel, 99)),
        mean_rel=float(abs(lum_g.mean() - lum_o.mean()) / max(lum_o.mean(), 1e-12)),
    )
    return out
