"""st_render_frames_noalloc: the camera-track render for callers that cannot
allocate device memory (engine-owned memory pools, real-time loops with a
fixed memory budget that cannot take the device-wide synchronisation of an
allocation).

The caller owns every buffer it passes (here torch allocates them, as the
calling application would); the library's working memory is its fixed
device array.  The output must match the regular entry point
(st_render_frames, which allocates through its context) on two calls in a
row, within the tolerance of the FP32 parity tests (relative 1e-5).
This file is collected last so a failure here cannot hide the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from spacetime_gb300 import _abi, api, workloads
from spacetime_gb300.api import Context, _st_camera, _st_spacetime

pytestmark = pytest.mark.gpu


def _device_inputs(sky_rgb, vol):
    import torch
    h, w, _ = sky_rgb.shape
    rgba = np.zeros((h, w, 4), np.float32)
    rgba[..., :3] = sky_rgb
    sky_d = torch.from_numpy(rgba).cuda()
    dens_d = torch.from_numpy(np.ascontiguousarray(vol.density)).cuda() if vol is not None else None
    return sky_d, dens_d


def _noalloc(lib, sky_d, sky_w, sky_h, disc, dens_d, vol, cams, bh, p, out_d):
    import torch
    cams_c = (_abi.StCamera * len(cams))(*[_st_camera(c) for c in cams])
    stats = _abi.StStats()
    dv = None
    if vol is not None:
        nr, nphi, nz = vol.shape
        dv = _abi.StVolume(None, nr, nphi, nz, vol.log_s_in, vol.log_s_out, vol.z_max, vol.emission_scale,
                           vol.opacity_scale, vol.march_stride)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.st_render_frames_noalloc(C.c_void_p(sky_d.data_ptr()), sky_w, sky_h, C.byref(disc) if disc else None,
                                      C.c_void_p(dens_d.data_ptr()) if dens_d is not None else None,
                                      C.byref(dv) if dv is not None else None, len(cams), cams_c,
                                      C.byref(_st_spacetime(bh)), C.byref(p), C.c_void_p(out_d.data_ptr()),
                                      C.c_void_p(stream), C.byref(stats))
    return rc, stats


@pytest.mark.parametrize("case", ["freefall_thin_disc", "kerr_gas"])
def test_noalloc_matches_regular_entry_point(built_lib, case):
    import torch
    lib = _abi.load()
    if case == "freefall_thin_disc":
        w = workloads.config2(nframes=6, width=96, height=54)
        cams, W, H = w.cams[::2], 96, 54
    else:
        w = workloads.config1(nr=64, nphi=32, nz=16)
        cams, W, H = [w.cam, w.cam], 120, 68
    sky = workloads.sky(512, 256)
    with Context(sky, disc=w.disc, volume=w.vol, emitter=w.emitter) as ctx:
        p = ctx.params(_abi.ST_SEM_DRAFT, width=W, height=H, samples=1, pixel_jitter=0,
                       precision=_abi.ST_PREC_FP32, schedule=_abi.ST_SCHED_PERSISTENT,
                       exit_landing=1, nmax=w.params.get("nmax", 0))
        ref = ctx.render_frames_raw(cams, w.bh, p)
    bb = w.disc.blackbody
    disc = _abi.StDisc(w.disc.inner_radius, w.disc.outer_radius, w.disc.density_falloff, bb.wb_temperature,
                       bb.table_min, bb.table_max, bb.table_size, w.emitter)
    if w.vol is not None:
        disc.inner = 0.0  # the gas replaces the thin plane, as in the context path
    sky_d, dens_d = _device_inputs(sky, w.vol)
    out_d = torch.zeros((len(cams), H, W, 4), dtype=torch.float32, device="cuda")
    for call in range(2):
        out_d.fill_(-1.0)
        rc, stats = _noalloc(lib, sky_d, sky.shape[1], sky.shape[0], disc, dens_d, w.vol, cams, w.bh, p, out_d)
        assert rc == _abi.ST_OK, lib.st_strerror(rc)
        assert stats.rays == len(cams) * W * H
        got = out_d[..., :3].cpu().numpy()
        np.testing.assert_allclose(got, ref.image, rtol=1e-5, atol=1e-7)
        assert stats.steps == ref.stats["steps"]


def test_noalloc_rejects_over_capacity(built_lib):
    import torch
    lib = _abi.load()
    w = workloads.config2(nframes=2, width=16, height=8)
    sky = workloads.sky(512, 256)
    sky_d, _ = _device_inputs(sky, None)
    p = _abi.StRenderParams()
    lib.st_render_params_default(C.byref(p), _abi.ST_SEM_DRAFT)
    p.width, p.height, p.samples = 16, 8, 1
    cams = [w.cams[0]] * 65
    out_d = torch.zeros((65, 8, 16, 4), dtype=torch.float32, device="cuda")
    rc, _ = _noalloc(lib, sky_d, sky.shape[1], sky.shape[0], None, None, None, cams, w.bh, p, out_d)
    assert rc == _abi.ST_ELIMIT
    assert b"scratch" in lib.st_strerror(rc)


def test_noalloc_rejects_what_the_context_path_rejects(built_lib):
    """The argument checks of st_render_frames and the context setters: an
    unknown emitter or an empty gas extent is ST_EINVAL, the surrogate and the
    adaptive integrators are ST_EUNSUPPORTED -- all before any device work."""
    import torch
    lib = _abi.load()
    w = workloads.config1(nr=8, nphi=4, nz=4)
    sky = workloads.sky(512, 256)
    sky_d, dens_d = _device_inputs(sky, w.vol)
    out_d = torch.zeros((1, 8, 16, 4), dtype=torch.float32, device="cuda")
    bb = w.disc.blackbody

    def params(**kw):
        p = _abi.StRenderParams()
        lib.st_render_params_default(C.byref(p), _abi.ST_SEM_DRAFT)
        p.width, p.height, p.samples = 16, 8, 1
        p.precision = _abi.ST_PREC_FP32
        for k, v in kw.items():
            setattr(p, k, v)
        return p

    def disc(emitter):
        return _abi.StDisc(0.0, w.disc.outer_radius, 0.0, bb.wb_temperature, bb.table_min, bb.table_max,
                           bb.table_size, emitter)

    ok = disc(w.emitter)
    assert _noalloc(lib, sky_d, 512, 256, disc(7), dens_d, w.vol, [w.cam], w.bh, params(), out_d)[0] == _abi.ST_EINVAL
    assert _noalloc(lib, sky_d, 512, 256, ok, dens_d, w.vol, [w.cam], w.bh, params(surrogate=1),
                    out_d)[0] == _abi.ST_EUNSUPPORTED
    assert _noalloc(lib, sky_d, 512, 256, ok, dens_d, w.vol, [w.cam], w.bh, params(order=45),
                    out_d)[0] == _abi.ST_EUNSUPPORTED
    bad = w.vol.__class__(**{**w.vol.__dict__, "z_max": 0.0})
    assert _noalloc(lib, sky_d, 512, 256, ok, dens_d, bad, [w.cam], w.bh, params(), out_d)[0] == _abi.ST_EINVAL
    bad = w.vol.__class__(**{**w.vol.__dict__, "log_s_out": w.vol.log_s_in})
    assert _noalloc(lib, sky_d, 512, 256, ok, dens_d, bad, [w.cam], w.bh, params(), out_d)[0] == _abi.ST_EINVAL
    # and a valid call still works afterwards
    rc, stats = _noalloc(lib, sky_d, 512, 256, ok, dens_d, w.vol, [w.cam], w.bh, params(), out_d)
    assert rc == _abi.ST_OK and stats.rays == 16 * 8
