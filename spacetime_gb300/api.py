"""Python host API over the C ABI, mirroring SpaceTime.jl's render interface.

    Schwarzschild(M), Kerr(M, a)                 src/gr.jl:7-34
    Blackbody(...), AccretionDisc(...)           src/blackbody.jl:42-60, src/accretion_disc.jl:5-13
    Lens(f), Camera                              src/raytrace.jl:22-29, src/camera.jl:36-50
    render(cam, bh, sky; disc, width, height)    src/raytrace.jl:339-428
    Context(sky; disc, volume)                   MetalPreviewContext, src/metal.jl:129-182
    render_draft(ctx, cam, bh; ...)              render_draft_mtl, src/metal.jl:2040-2242
    render_depth(ctx, cam, bh; nbuckets, ...)    render_depth_mtl, src/metal.jl:1935-1990
    DiscFluidSim(ctx, vol, disc), step_sim       src/disc_sim.jl:38-91, 280-320

Images come back as float32 arrays of shape (height, width, 3): element
[j, i] is pixel (i, j) of the reference's Matrix{RGBf}(width, height), i.e.
the same bytes as its column-major (3, width, height) buffer.  Row j = 0 is
the bottom of the frame.  Every call runs the CUDA library; there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .scene import Camera, Volume, lens_fov

__all__ = [
    "Schwarzschild", "Kerr", "Blackbody", "AccretionDisc", "Lens", "Camera", "Context",
    "render", "render_draft", "render_depth", "render_frames", "camera_tetrad", "RenderResult",
    "DiscFluidSim", "step_sim",
]


@dataclass(frozen=True)
class Schwarzschild:
    M: float = 1.0

    @property
    def a(self) -> float:
        return 0.0


@dataclass(frozen=True)
class Kerr:
    M: float
    a: float

    def __post_init__(self):
        if not abs(self.a) <= self.M:
            # src/gr.jl:31: ArgumentError("|a| must be <= M")
            raise ValueError(f"|a| must be <= M (got a={self.a}, M={self.M})")


@dataclass(frozen=True)
class Blackbody:
    wb_temperature: float = 6500.0
    table_min: float = 500.0
    table_max: float = 30000.0
    table_size: int = 1024


@dataclass(frozen=True)
class AccretionDisc:
    inner_radius: float = 3.0
    outer_radius: float = 20.0
    blackbody: Blackbody = field(default_factory=Blackbody)
    density_falloff: float = 0.0


@dataclass(frozen=True)
class Lens:
    focal_length: float

    @property
    def fov_factor(self) -> float:
        return lens_fov(self.focal_length)


@dataclass(frozen=True)
class Starfield:
    """Procedural point stars, Starfield(...) of the CPU renderer
    (src/starfield.jl:60-81) and set_starfield!(ctx; ...) of the GPU one
    (src/metal.jl:257-295), argument for argument."""
    strength: float = 1.0
    texture_weight: float = 0.0
    height: int = 1080
    fov_factor: float = 0.55
    density: float = 384.0
    fill: float = 0.5
    flux: float = 0.011
    psf_pixels: float = 0.5
    galactic: tuple = (0.0, 0.0, 1.0)
    concentration: float = 3.0
    temp_min: float = 3000.0
    temp_max: float = 16000.0
    seed: int = 12345
    wb_temperature: float = 10000.0
    saturation: float = 1.0
    table_size: int = 1024

    def as_c(self) -> "_abi.StStarfield":
        c = _abi.StStarfield()
        for name, _ in _abi.StStarfield._fields_:
            v = getattr(self, name)
            if name == "galactic":
                c.galactic[:] = [float(x) for x in v]
            else:
                setattr(c, name, v)
        return c


@dataclass
class RenderResult:
    image: np.ndarray
    stats: dict
    diag: np.ndarray | None = None


def _st_camera(cam: Camera) -> _abi.StCamera:
    c = _abi.StCamera()
    c.pos[:] = [float(v) for v in cam.pos]
    c.fwd[:] = [float(v) for v in cam.fwd]
    c.right[:] = [float(v) for v in cam.right]
    c.up[:] = [float(v) for v in cam.up_local]
    c.fov_factor = float(cam.fov_factor)
    c.velocity[:] = [float(v) for v in cam.velocity]
    c.projection = int(cam.projection)
    c.fisheye_deg = float(cam.fisheye_deg)
    c.aperture_world = float(cam.aperture_world)
    c.focus_dist = float(cam.focus_dist)
    return c


def _st_spacetime(bh) -> _abi.StSpacetime:
    return _abi.StSpacetime(float(bh.M), float(getattr(bh, "a", 0.0)))


def camera_tetrad(cam: Camera, bh) -> np.ndarray:
    """(u, Ef, Er, Eu) as a 4x4 array (rows), src/preview.jl:93-198."""
    lib = _abi.load()
    out = (C.c_double * 16)()
    _abi.check(lib.st_camera_tetrad(C.byref(_st_camera(cam)), C.byref(_st_spacetime(bh)), out),
               "st_camera_tetrad")
    return np.array(out[:]).reshape(4, 4)


class Context:
    """Device-resident sky, blackbody table and gas grid (MetalPreviewContext)."""

    def __init__(self, sky: np.ndarray, disc: AccretionDisc | None = None, volume: Volume | None = None,
                 emitter: int | None = None, device: int = 0):
        self._lib = _abi.load()
        sky = np.ascontiguousarray(sky, dtype=np.float32)
        if sky.ndim != 3 or sky.shape[2] != 3:
            raise ValueError("sky must be (height, width, 3) float32")
        h, w, _ = sky.shape
        handle = C.c_void_p()
        _abi.check(self._lib.st_context_create(C.byref(handle), sky.ctypes.data_as(C.POINTER(C.c_float)),
                                               w, h, device), "st_context_create")
        self._h = handle
        self.sky_shape = (w, h)
        self.disc = None
        self.volume = None
        self.emitter = emitter
        self.set_disc(disc, emitter)
        self.set_volume(volume)

    def set_disc(self, disc: AccretionDisc | None, emitter: int | None = None):
        if disc is None:
            _abi.check(self._lib.st_context_set_disc(self._h, None), "st_context_set_disc")
            self.disc = None
            return
        bb = disc.blackbody
        em = _abi.ST_EMIT_KS_EXACT if emitter is None else emitter
        d = _abi.StDisc(disc.inner_radius, disc.outer_radius, disc.density_falloff, bb.wb_temperature,
                        bb.table_min, bb.table_max, bb.table_size, em)
        _abi.check(self._lib.st_context_set_disc(self._h, C.byref(d)), "st_context_set_disc")
        self.disc = disc
        self.emitter = em

    def set_volume(self, vol: Volume | None):
        if vol is None:
            _abi.check(self._lib.st_context_set_volume(self._h, None), "st_context_set_volume")
            self.volume = None
            return
        dens = np.ascontiguousarray(vol.density, dtype=np.float32)
        nr, nphi, nz = vol.shape
        v = _abi.StVolume(dens.ctypes.data_as(C.POINTER(C.c_float)), nr, nphi, nz, vol.log_s_in,
                          vol.log_s_out, vol.z_max, vol.emission_scale, vol.opacity_scale, vol.march_stride)
        _abi.check(self._lib.st_context_set_volume(self._h, C.byref(v)), "st_context_set_volume")
        self.volume = vol

    def set_starfield(self, sf: Starfield | None = None, **kw):
        """set_starfield!(ctx; strength, texture_weight, height, fov_factor,
        density, fill, flux, psf_pixels, galactic, concentration, temp_min,
        temp_max, seed, wb_temperature, saturation): a Starfield, or its
        fields as keywords; None (or strength 0) turns the stars off."""
        if sf is None and kw:
            sf = Starfield(**kw)
        c = sf.as_c() if sf is not None else None
        _abi.check(self._lib.st_context_set_starfield(self._h, C.byref(c) if c is not None else None),
                   "st_context_set_starfield")
        self.starfield = sf

    def set_surrogate(self, sur):
        """Attach a trained surrogate (spacetime_gb300.surrogate.Surrogate) for
        renders with surrogate=1; None detaches it."""
        _abi.check(self._lib.st_context_set_surrogate(self._h, sur._h if sur is not None else None),
                   "st_context_set_surrogate")
        self._sur = sur

    def close(self):
        if getattr(self, "_h", None):
            self._lib.st_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- low level ------------------------------------------------------------
    def params(self, semantics: int, **kw) -> _abi.StRenderParams:
        p = _abi.StRenderParams()
        self._lib.st_render_params_default(C.byref(p), semantics)
        for k, v in kw.items():
            if not hasattr(p, k):
                raise TypeError(f"unknown render parameter {k!r}")
            setattr(p, k, v)
        return p

    def render_raw(self, cam: Camera, bh, p: _abi.StRenderParams, diag: bool = False,
                   out: np.ndarray | None = None) -> RenderResult:
        img = out if out is not None else np.empty((p.height, p.width, 3), dtype=np.float32)
        stats = _abi.StStats()
        cam_c, st_c = _st_camera(cam), _st_spacetime(bh)
        fptr = img.ctypes.data_as(C.POINTER(C.c_float))
        if diag:
            d = np.empty(p.height * p.width, dtype=_abi.DIAG_DTYPE)
            rc = self._lib.st_render_diag(self._h, C.byref(cam_c), C.byref(st_c), C.byref(p), fptr,
                                          C.c_void_p(d.ctypes.data), C.byref(stats))
            _abi.check(rc, "st_render_diag")
            return RenderResult(img, stats.as_dict(), d.reshape(p.height, p.width))
        rc = self._lib.st_render(self._h, C.byref(cam_c), C.byref(st_c), C.byref(p), fptr, C.byref(stats))
        _abi.check(rc, "st_render")
        return RenderResult(img, stats.as_dict())

    def render_device(self, cam: Camera, bh, p: _abi.StRenderParams) -> tuple[int, dict]:
        """Render, leaving the float4 frame on the device; returns its address."""
        stats = _abi.StStats()
        ptr = C.c_void_p()
        rc = self._lib.st_render_device(self._h, C.byref(_st_camera(cam)), C.byref(_st_spacetime(bh)),
                                        C.byref(p), C.byref(ptr), C.byref(stats))
        _abi.check(rc, "st_render_device")
        return ptr.value, stats.as_dict()

    def render_motion_raw(self, cam: Camera, poses, bh, p: _abi.StRenderParams, per_pixel_shutter: bool = False,
                          diag: bool = False) -> RenderResult:
        """Motion-blurred render (st_render_motion): poses are camera_at
        sampled at (m + 1/2)/samples^2 (midpoint) or m/samples^2, m <=
        samples^2 (per-pixel shutter)."""
        n = len(poses)
        arr = (_abi.StCamera * n)(*[_st_camera(c) for c in poses])
        img = np.empty((p.height, p.width, 3), dtype=np.float32)
        d = np.empty(p.height * p.width, dtype=_abi.DIAG_DTYPE) if diag else None
        stats = _abi.StStats()
        rc = self._lib.st_render_motion(self._h, C.byref(_st_camera(cam)), arr, n, int(per_pixel_shutter),
                                        C.byref(_st_spacetime(bh)), C.byref(p),
                                        img.ctypes.data_as(C.POINTER(C.c_float)),
                                        C.c_void_p(d.ctypes.data) if diag else None, C.byref(stats))
        _abi.check(rc, "st_render_motion")
        return RenderResult(img, stats.as_dict(), d.reshape(p.height, p.width) if diag else None)

    def sky_fan(self, cam: Camera, bh, p: _abi.StRenderParams):
        """(fan (4096, 4), fine (1024, 4), band (2,)) for this camera
        (update_sky_fan!): columns escaped, cos, sin of the exit angle from the
        radial axis, periapsis."""
        fan = np.empty((_abi.ST_FAN_N, 4), np.float32)
        fine = np.empty((_abi.ST_FAN_FINE, 4), np.float32)
        band = np.empty(2, np.float32)
        fp = C.POINTER(C.c_float)
        _abi.check(self._lib.st_sky_fan(self._h, C.byref(_st_camera(cam)), C.byref(_st_spacetime(bh)), C.byref(p),
                                        fan.ctypes.data_as(fp), fine.ctypes.data_as(fp), band.ctypes.data_as(fp)),
                   "st_sky_fan")
        return fan, fine, band

    def render_layered_raw(self, cam: Camera, bh, p: _abi.StRenderParams, layer_size=None,
                           diag: bool = False, ring_rmin: float = 0.0, ring_size=None,
                           ring_box: bool = True) -> RenderResult:
        """The layered engine's frame (render_layered_gpu!): fan-driven sky,
        disc / gas layer at layer_size = (width, height) (default: the display);
        ring_rmin > 0 adds the foveated ring pass at ring_size (default: the
        display) for rays whose fan periapsis is below ring_rmin."""
        lw, lh = layer_size if layer_size is not None else (0, 0)
        img = np.empty((p.height, p.width, 3), dtype=np.float32)
        d = np.empty(p.height * p.width, dtype=_abi.DIAG_DTYPE) if diag else None
        stats = _abi.StStats()
        args = (self._h, C.byref(_st_camera(cam)), C.byref(_st_spacetime(bh)), C.byref(p), int(lw), int(lh))
        tail = (img.ctypes.data_as(C.POINTER(C.c_float)), C.c_void_p(d.ctypes.data) if diag else None,
                C.byref(stats))
        if ring_rmin > 0:
            rw, rh = ring_size if ring_size is not None else (0, 0)
            _abi.check(self._lib.st_render_layered_ring(*args, int(rw), int(rh), float(ring_rmin), int(ring_box),
                                                        *tail), "st_render_layered_ring")
        else:
            _abi.check(self._lib.st_render_layered(*args, *tail), "st_render_layered")
        return RenderResult(img, stats.as_dict(), d.reshape(p.height, p.width) if diag else None)

    def render_depth_raw(self, cam: Camera, bh, p: _abi.StRenderParams, nbuckets: int = 10) -> RenderResult:
        """Depth-bucketed frame (st_render_depth): image has shape
        (height, width, nbuckets, 3); bucket nbuckets - 1 is the sky."""
        img = np.empty((p.height, p.width, nbuckets, 3), dtype=np.float32)
        stats = _abi.StStats()
        _abi.check(self._lib.st_render_depth(self._h, C.byref(_st_camera(cam)), C.byref(_st_spacetime(bh)),
                                             C.byref(p), int(nbuckets), img.ctypes.data_as(C.POINTER(C.c_float)),
                                             C.byref(stats)),
                   "st_render_depth")
        return RenderResult(img, stats.as_dict())

    def render_frames_raw(self, cams, bh, p: _abi.StRenderParams) -> RenderResult:
        n = len(cams)
        arr = (_abi.StCamera * n)(*[_st_camera(c) for c in cams])
        img = np.empty((n, p.height, p.width, 3), dtype=np.float32)
        stats = _abi.StStats()
        rc = self._lib.st_render_frames(self._h, n, arr, C.byref(_st_spacetime(bh)), C.byref(p),
                                        img.ctypes.data_as(C.POINTER(C.c_float)), C.byref(stats))
        _abi.check(rc, "st_render_frames")
        return RenderResult(img, stats.as_dict())


_PREC = {"fp64": _abi.ST_PREC_FP64, "fp32": _abi.ST_PREC_FP32, "fp32g": _abi.ST_PREC_FP32_GUARDED,
         "fp32_guarded": _abi.ST_PREC_FP32_GUARDED, "fp32g_df": _abi.ST_PREC_FP32_GUARDED_DF,
         "fp32_guarded_df": _abi.ST_PREC_FP32_GUARDED_DF}


def _prec(x):
    return _PREC[x] if isinstance(x, str) else int(x)


def render(cam: Camera, bh, sky: np.ndarray, *, disc: AccretionDisc | None = AccretionDisc(),
           width: int = 400, height: int = 200, samples: int = 1, relativistic: bool = False,
           precision="fp64", dt: float = 0.02, jittered: bool = False, seed: int = 0,
           starfield: Starfield | None = None, context: Context | None = None, **kw) -> np.ndarray:
    """The CPU renderer's call, `render(cam, bh, sky; disc, width, height,
    samples, relativistic)` (src/raytrace.jl:339-428), on the GPU: horizon at
    r = 2.00001, escape at r_max = max(5|pos|, 100), affine budget
    max(10|pos|, 500), Keplerian Planck-Doppler disc, black iff r < 2.1M.
    `jittered=False` places samples at stratum centres (the reference's
    `jittered=false`); jittered samples are hashed per pixel, not drawn from
    Julia's Xoshiro stream."""
    if not isinstance(bh, Schwarzschild) and getattr(bh, "a", 0.0) != 0.0:
        # the reference has no render(cam, ::Kerr, ...) method
        raise TypeError("render: the CPU-renderer semantics are Schwarzschild-only; use render_draft")
    ctx = context or Context(sky, disc=disc, emitter=_abi.ST_EMIT_KEPLER)
    if starfield is not None or context is None:
        ctx.set_starfield(starfield)
    try:
        p = ctx.params(_abi.ST_SEM_RENDER, width=width, height=height, samples=samples,
                       relativistic=int(relativistic), precision=_prec(precision), dt=dt,
                       pixel_jitter=int(jittered), seed=seed, **kw)
        return ctx.render_raw(cam, bh, p).image
    finally:
        if context is None:
            ctx.close()


def render_draft(ctx: Context, cam: Camera, bh, *, width: int = 1920, height: int = 1080, samples: int = 2,
                 dt: float = 0.02, fisheye_deg: float = 0.0, aperture_world: float = 0.0,
                 focus_dist: float = 1.0, relativistic: bool = False, precision="fp32",
                 pixel_jitter: bool = True, seed: int = 0, camera_at=None, per_pixel_shutter: bool = False,
                 **kw) -> np.ndarray:
    """render_draft_mtl(ctx, cam, st; width, height, samples, dt, fisheye_deg,
    aperture_world, focus_dist, relativistic, camera_at, per_pixel_shutter)
    (src/metal.jl:2040-2242).  camera_at(s) -> Camera for the shutter
    fraction s in [0, 1) turns on motion blur."""
    cam2 = Camera(cam.pos, cam.fwd, cam.right, cam.up_local, cam.fov_factor, cam.velocity,
                  _abi.ST_PROJ_FISHEYE if fisheye_deg > 0 else _abi.ST_PROJ_PINHOLE, fisheye_deg,
                  aperture_world, focus_dist)
    p = ctx.params(_abi.ST_SEM_DRAFT, width=width, height=height, samples=samples, dt=dt,
                   relativistic=int(relativistic), precision=_prec(precision),
                   pixel_jitter=int(pixel_jitter), seed=seed, **kw)
    if camera_at is not None:
        n = samples * samples
        poses = ([camera_at(m / n) for m in range(n + 1)] if per_pixel_shutter
                 else [camera_at((m + 0.5) / n) for m in range(n)])
        return ctx.render_motion_raw(cam2, poses, bh, p, per_pixel_shutter=per_pixel_shutter).image
    return ctx.render_raw(cam2, bh, p).image


def render_depth(ctx: Context, cam: Camera, bh, *, width: int = 1920, height: int = 1080, samples: int = 2,
                 dt: float = 0.02, nbuckets: int = 10, fisheye_deg: float = 0.0, relativistic: bool = False,
                 precision="fp32", seed: int = 0, **kw) -> np.ndarray:
    """render_depth_mtl(ctx, cam, st; width, height, samples, dt, nbuckets,
    fisheye_deg, relativistic) (src/metal.jl:1935-1990): a pinhole (or
    fisheye) draft frame with emission split into nbuckets path-length
    buckets, log-spaced over 1.5-120 M, the last holding the sky.  Returns
    (height, width, nbuckets, 3); summing over buckets gives the plain frame.
    Raises ValueError for nbuckets < 3, as the reference does."""
    if nbuckets < 3:
        raise ValueError("nbuckets must be >= 3")
    cam2 = Camera(cam.pos, cam.fwd, cam.right, cam.up_local, cam.fov_factor, cam.velocity,
                  _abi.ST_PROJ_FISHEYE if fisheye_deg > 0 else _abi.ST_PROJ_PINHOLE, fisheye_deg, 0.0, 1.0)
    kw.setdefault("pixel_jitter", 0)
    p = ctx.params(_abi.ST_SEM_DRAFT, width=width, height=height, samples=samples, dt=dt,
                   relativistic=int(relativistic), precision=_prec(precision), seed=seed, **kw)
    return ctx.render_depth_raw(cam2, bh, p, nbuckets).image


class DiscFluidSim:
    """DiscFluidSim(ctx, vol, disc; M, forcing, drag, relax) (src/disc_sim.jl:38-91):
    the live fluid disc on the context volume's grid.  step() is step_sim!
    (src/disc_sim.jl:280-320): it advances the solver and writes the extruded
    density into the context's gas texture, so the next render sees it.  vol
    is the Volume the context holds (for its scale height).  Fields come back
    as (nphi, nr) float32 arrays (the reference's (nr, nphi) column-major)."""

    def __init__(self, ctx: Context, vol: Volume, disc: AccretionDisc, *, M: float = 1.0, forcing: float = 6.0,
                 drag: float = 0.15, relax: float = 0.05):
        if ctx.volume is None:
            raise ValueError("the context holds no volume")
        self._lib = ctx._lib
        self.ctx = ctx                     # the solver writes into this context's texture
        self.shape = vol.shape
        fp = _abi.StFluidParams(M, forcing, drag, relax, vol.scale_height)
        bb = disc.blackbody
        d = _abi.StDisc(disc.inner_radius, disc.outer_radius, disc.density_falloff, bb.wb_temperature,
                        bb.table_min, bb.table_max, bb.table_size, _abi.ST_EMIT_KS_EXACT)
        h = C.c_void_p()
        _abi.check(self._lib.st_fluid_create(C.byref(h), ctx._h, C.byref(d), C.byref(fp)), "st_fluid_create")
        self._h = h

    def step(self, dt: float = 0.05, jacobi: int = 8, nsteps: int = 1, graph: bool = True,
             timed: bool = False) -> float | None:
        """nsteps solver steps; timed=True waits and returns their device ms."""
        ms = C.c_float(0.0)
        _abi.check(self._lib.st_fluid_step(self._h, float(dt), int(jacobi), int(nsteps), int(graph),
                                           C.byref(ms) if timed else None), "st_fluid_step")
        return float(ms.value) if timed else None

    def state(self, volume: bool = False) -> dict:
        nr, nphi, nz = self.shape
        out = {k: np.empty((nphi, nr), np.float32) for k in ("vu", "vv", "dens")}
        vol = np.empty((nz, nphi, nr), np.float32) if volume else None
        t = C.c_double(0.0)
        fp = C.POINTER(C.c_float)
        _abi.check(self._lib.st_fluid_state(self._h, out["vu"].ctypes.data_as(fp), out["vv"].ctypes.data_as(fp),
                                            out["dens"].ctypes.data_as(fp),
                                            vol.ctypes.data_as(fp) if volume else None, C.byref(t)),
                   "st_fluid_state")
        out["t"] = t.value
        if volume:
            out["volume"] = vol
        return out

    def close(self):
        if getattr(self, "_h", None):
            self._lib.st_fluid_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def step_sim(sim: DiscFluidSim, ctx: Context | None = None, *, dt: float = 0.05, jacobi: int = 8) -> None:
    """step_sim!(sim, ctx; dt, jacobi) (src/disc_sim.jl:287-320)."""
    if ctx is not None and ctx is not sim.ctx:
        raise ValueError("the solver writes into the context it was built on")
    sim.step(dt=dt, jacobi=jacobi)


def render_frames(ctx: Context, cams, bh, *, width: int, height: int, dt: float = 0.02, precision="fp32g",
                  **kw) -> np.ndarray:
    """A camera track rendered in one persistent launch (DRAFT semantics)."""
    p = ctx.params(_abi.ST_SEM_DRAFT, width=width, height=height, samples=1, dt=dt,
                   precision=_prec(precision), pixel_jitter=0, schedule=_abi.ST_SCHED_PERSISTENT, **kw)
    return ctx.render_frames_raw(cams, bh, p).image
