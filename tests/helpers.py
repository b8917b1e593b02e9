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


# ---- the host's pass plan, restated (st_api.cu plan_passes) -----------------
_M64 = (1 << 64) - 1


class _SplitMix64:
    def __init__(self, s):
        self.s = s & _M64

    def next(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & _M64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)

    def below(self, n):
        return self.next() % n


def _shuffle(v, rng):
    for i in range(len(v) - 1, 0, -1):
        k = rng.below(i + 1)
        v[i], v[k] = v[k], v[i]


def pass_plan(samples, seed, pixel_jitter, semantics, dof, block=0):
    """The samples^2 passes of one render as the host plans them: per pass
    the pixel stratum (ju, jv, jw, jseed) and the lens stratum (lens_u0,
    lens_v0, lens_w, lens_seed; zeros without depth of field), in launch
    order.  Seeded splitmix64 shuffles, as render_draft_mtl shuffles its
    strata (src/metal.jl:2091-2168)."""
    S = samples
    n = S * S
    rng = _SplitMix64(((seed ^ 0x5EED5EED) + 0x9E3779B97F4A7C15 * block) & _M64)
    order, lens, tperm = list(range(n)), list(range(n)), list(range(n))
    if pixel_jitter:
        _shuffle(order, rng)
    _shuffle(lens, rng)
    _shuffle(tperm, rng)
    shift = 0.5 if semantics == _abi.ST_SEM_RENDER else 0.0
    out = []
    for k in range(n):
        m = order[k]
        a, b = m // S, m % S
        if pixel_jitter:
            ju, jv, jw = a / S + shift, b / S + shift, 1.0 / S
        else:
            ju, jv, jw = (a + 0.5) / S + shift, (b + 0.5) / S + shift, 0.0
        pss = block * n + k + 1
        pp = dict(ju=ju, jv=jv, jw=jw, jseed=15485863 + pss, lens_u0=0.0, lens_v0=0.0, lens_w=0.0, lens_seed=0)
        if dof:
            lm = lens[k]
            pp.update(lens_u0=(lm // S) / S, lens_v0=(lm % S) / S, lens_w=1.0 / S, lens_seed=pss)
        out.append(pp)
    return out


def oracle_pass(scene, pp, aperture_radius=0.0):
    """Set one planned pass's strata on an oracle scene."""
    s = scene.s
    s.ju, s.jv, s.jitter_w, s.jitter_seed = pp["ju"], pp["jv"], pp["jw"], pp["jseed"]
    s.aperture_radius = aperture_radius
    s.lens_u0, s.lens_v0, s.lens_w, s.lens_seed = pp["lens_u0"], pp["lens_v0"], pp["lens_w"], pp["lens_seed"]
    return scene
