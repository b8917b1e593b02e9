"""ctypes wrapper of the FP64 oracle (oracle/st_oracle.cpp).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  The product never imports it.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libst_oracle.so")

SEM_RENDER, SEM_DRAFT = 0, 1
INT_RK4, INT_TSIT5, INT_TSIT5_K45, INT_TSIT5_K46 = 0, 1, 2, 3
EMIT_KEPLER, EMIT_KS_EXACT = 0, 1
RAY_ESCAPED, RAY_CAPTURED, RAY_BUDGET, RAY_BLACK, RAY_CROSSED, RAY_GRAZE, RAY_BCAPT = 1, 2, 4, 8, 16, 32, 64

D3 = C.c_double * 3
FP = C.POINTER(C.c_float)


class OrcScene(C.Structure):
    _fields_ = [
        ("pos", D3), ("fwd", D3), ("right", D3), ("up", D3), ("fov", C.c_double), ("velocity", D3),
        ("projection", C.c_int), ("fisheye_rad", C.c_double), ("aperture_radius", C.c_double),
        ("focus_dist", C.c_double), ("lens_seed", C.c_int), ("lens_u0", C.c_double), ("lens_v0", C.c_double),
        ("lens_w", C.c_double),
        ("M", C.c_double), ("a", C.c_double),
        ("disc_on", C.c_int), ("disc_inner", C.c_double), ("disc_outer", C.c_double),
        ("disc_falloff", C.c_double), ("emitter", C.c_int), ("bb_lut", FP), ("lut_size", C.c_int),
        ("lut_tmin", C.c_double), ("lut_tmax", C.c_double),
        ("vol_on", C.c_int), ("vol", FP), ("nr", C.c_int), ("nphi", C.c_int), ("nz", C.c_int),
        ("vol_ls_in", C.c_double), ("vol_ls_out", C.c_double), ("vol_zmax", C.c_double),
        ("vol_emis", C.c_double), ("vol_opac", C.c_double), ("vol_stride", C.c_int),
        ("sky", FP), ("sky_w", C.c_int), ("sky_h", C.c_int),
        ("width", C.c_int), ("height", C.c_int), ("col0", C.c_int), ("cols", C.c_int), ("row0", C.c_int),
        ("rows", C.c_int), ("ju", C.c_double), ("jv", C.c_double), ("jitter_w", C.c_double),
        ("jitter_seed", C.c_int),
        ("semantics", C.c_int), ("integrator", C.c_int), ("dt", C.c_double), ("nmax", C.c_int),
        ("r_escape", C.c_double), ("tspan", C.c_double), ("hstep_coef", C.c_double),
        ("hstep_cap", C.c_double), ("rtol", C.c_double), ("atol", C.c_double), ("relativistic", C.c_int),
        ("exit_landing", C.c_int), ("tol", C.c_double),
        ("shutter_seed", C.c_int), ("pos_end", D3), ("u_end", C.c_double * 4), ("Ef_end", C.c_double * 4),
        ("Er_end", C.c_double * 4), ("Eu_end", C.c_double * 4),
        ("star_strength", C.c_double), ("star_tw", C.c_double), ("star_N", C.c_double), ("star_fill", C.c_double),
        ("star_sigma", C.c_double), ("star_flux", C.c_double), ("star_g", D3), ("star_conc", C.c_double),
        ("star_tmin", C.c_double), ("star_tspan", C.c_double), ("star_lut", FP), ("star_lut_size", C.c_int),
        ("star_seed", C.c_int), ("star_lut_tmin", C.c_double), ("star_lut_tmax", C.c_double),
    ]


RAY_DTYPE = np.dtype([
    ("dir", "<f8", (3,)), ("r_final", "<f8"), ("alpha", "<f8"), ("r_cross", "<f8"), ("g_cross", "<f8"),
    ("rgb", "<f8", (3,)), ("lambda_", "<f8"), ("flags", "<i4"), ("steps", "<i4"), ("rhs_evals", "<i4"),
    ("pad", "<i4"),
])

class OrcFluid(C.Structure):
    _fields_ = [("nr", C.c_int), ("nphi", C.c_int), ("nz", C.c_int),
                ("vu", FP), ("vv", FP), ("dens", FP), ("base", FP), ("env", FP), ("shear", FP),
                ("t", C.c_float), ("forcing", C.c_double), ("drag", C.c_double), ("relax", C.c_double)]


_lib = None


def build() -> str:
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        P = C.POINTER
        dp = P(C.c_double)
        L.orc_render.argtypes = [P(OrcScene), FP, C.c_void_p, C.c_int]
        L.orc_render.restype = C.c_int
        L.orc_fluid_init.argtypes = [P(OrcFluid), FP, C.c_float, C.c_float, C.c_float, C.c_double, C.c_double,
                                     C.c_double, C.c_double, C.c_double]
        L.orc_fluid_init.restype = C.c_int
        L.orc_fluid_step.argtypes = [P(OrcFluid), FP, C.c_double, C.c_int, C.c_int]
        L.orc_fluid_step.restype = C.c_int
        L.orc_render_depth.argtypes = [P(OrcScene), C.c_int, FP, C.c_int]
        L.orc_render_depth.restype = C.c_int
        L.orc_trace_dirs.argtypes = [P(OrcScene), C.c_int, P(C.c_double), C.c_void_p, C.c_int]
        L.orc_trace_dirs.restype = C.c_int
        L.orc_rhs.argtypes = [C.c_int, dp, C.c_double, C.c_double, C.c_double, dp]
        L.orc_camera_tetrad.argtypes = [dp, dp, dp, dp, C.c_double, C.c_double, dp, dp, dp, dp, dp]
        L.orc_camera_beta.argtypes = [dp, dp, dp, dp, dp]
        L.orc_init_photon.argtypes = [dp, dp, C.c_double, C.c_double, dp, dp]
        L.orc_metric.argtypes = [C.c_double, C.c_double, dp, dp]
        L.orc_metric_inverse.argtypes = [C.c_double, C.c_double, dp, dp]
        for n in ("orc_horizon_radius", "orc_photon_orbit_min"):
            getattr(L, n).argtypes = [C.c_double, C.c_double]
            getattr(L, n).restype = C.c_double
        L.orc_isco.argtypes = [C.c_double, C.c_double, dp]
        L.orc_blackbody_rgb.argtypes = [C.c_double, dp]
        L.orc_blackbody_lut.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int, FP]
        L.orc_sim_hash.argtypes = [C.c_int, C.c_int, C.c_int]
        L.orc_sim_hash.restype = C.c_float
        L.orc_shadow_radius.argtypes = [C.c_double, C.c_double, C.c_double]
        L.orc_shadow_radius.restype = C.c_double
        L.orc_lz_drift.argtypes = [C.c_double, C.c_double, C.c_int]
        L.orc_lz_drift.restype = C.c_double
        _lib = L
    return _lib


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


# ---- unit pieces -----------------------------------------------------------

def rhs(kerr: bool, s, pt, M, a):
    s, sp = _d(s)
    out = np.zeros(6)
    lib().orc_rhs(int(kerr), sp, pt, M, a, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def camera_tetrad(pos, fwd, right, up, M=1.0, a=0.0, beta=(0.0, 0.0, 0.0)):
    args = [_d(v) for v in (pos, fwd, right, up)]
    b = _d(beta)
    outs = [np.zeros(4) for _ in range(4)]
    lib().orc_camera_tetrad(*[x[1] for x in args], M, a, b[1],
                            *[o.ctypes.data_as(C.POINTER(C.c_double)) for o in outs])
    return tuple(outs)  # u, Ef, Er, Eu


def init_photon(origin, q, M=1.0, a=0.0):
    o, op = _d(origin)
    qq, qp = _d(q)
    s = np.zeros(6)
    pt = C.c_double()
    lib().orc_init_photon(op, qp, M, a, s.ctypes.data_as(C.POINTER(C.c_double)), C.byref(pt))
    return s, pt.value


def metric(M, a, x):
    xx, xp = _d(x)
    g = np.zeros(16)
    lib().orc_metric(M, a, xp, g.ctypes.data_as(C.POINTER(C.c_double)))
    return g.reshape(4, 4)


def metric_inverse(M, a, x):
    xx, xp = _d(x)
    g = np.zeros(16)
    lib().orc_metric_inverse(M, a, xp, g.ctypes.data_as(C.POINTER(C.c_double)))
    return g.reshape(4, 4)


def horizon_radius(M, a=0.0):
    return lib().orc_horizon_radius(M, a)


def photon_orbit_min(M, a=0.0):
    return lib().orc_photon_orbit_min(M, a)


def isco(M, a):
    out = np.zeros(3)
    lib().orc_isco(M, a, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def blackbody_lut(wb=6500.0, tmin=500.0, tmax=30000.0, n=1024):
    out = np.zeros((n, 3), dtype=np.float32)
    lib().orc_blackbody_lut(wb, tmin, tmax, n, out.ctypes.data_as(FP))
    return out


STAR_WB_TEMPERATURE = 10000.0  # src/metal.jl:75


def star_lut(wb=STAR_WB_TEMPERATURE, saturation=1.0, n=1024):
    """The stars' colour table (_star_lut_cpu, src/metal.jl:86-104): the
    white-balanced blackbody table over [500, 30000] K in float32, chroma
    scaled by `saturation` about Rec.709 luminance.  Shape (n, 3)."""
    lut = blackbody_lut(wb, 500.0, 30000.0, n).astype(np.float32)
    if saturation != 1.0:
        s = np.float32(saturation)
        L = (np.float32(0.2126) * lut[:, 0] + np.float32(0.7152) * lut[:, 1]
             + np.float32(0.0722) * lut[:, 2])[:, None]
        lut = (L + s * (lut - L)).astype(np.float32)
    return lut


def camera_beta_of(cam):
    """camera_beta (src/camera.jl:19-22): world velocity on the camera axes."""
    v = np.asarray(cam.velocity, dtype=np.float64)
    return (float(v @ cam.fwd), float(v @ cam.right), float(v @ cam.up_local))


def sim_hash(x, y, z):
    return lib().orc_sim_hash(x, y, z)


def shadow_radius(r_cam, M, fov):
    return lib().orc_shadow_radius(r_cam, M, fov)


def lz_drift(a, h=0.005, nmax=20000):
    return lib().orc_lz_drift(a, h, nmax)


# ---- full renders ----------------------------------------------------------

class Scene:
    """Keeps the numpy buffers alive alongside the C struct."""

    def __init__(self, *, cam, M, a, sky, width, height, semantics, integrator, dt=0.02, nmax=0,
                 r_escape=0.0, tspan=0.0, disc=None, emitter=EMIT_KEPLER, lut=None, volume=None,
                 relativistic=False, exit_landing=None, ju=None, jv=None, rtol=1e-10, atol=1e-12,
                 rect=None, tol=1e-4, starfield=None, shutter=None):
        s = OrcScene()
        s.pos[:] = list(map(float, cam.pos))
        s.fwd[:] = list(map(float, cam.fwd))
        s.right[:] = list(map(float, cam.right))
        s.up[:] = list(map(float, cam.up_local))
        s.fov = float(cam.fov_factor)
        s.velocity[:] = list(map(float, cam.velocity))
        s.projection = int(cam.projection)
        s.fisheye_rad = math.radians(max(cam.fisheye_deg, 0.0))
        s.focus_dist = float(cam.focus_dist) if cam.focus_dist > 0 else 1.0
        s.M, s.a = float(M), float(a)
        self._keep = []
        if disc is not None:
            s.disc_on = 1
            s.disc_inner, s.disc_outer, s.disc_falloff = disc["inner"], disc["outer"], disc.get("falloff", 0.0)
            s.emitter = emitter
            lut = np.ascontiguousarray(lut if lut is not None else blackbody_lut(disc.get("wb", 6500.0)),
                                       dtype=np.float32)
            self._keep.append(lut)
            s.bb_lut = lut.ctypes.data_as(FP)
            s.lut_size = lut.shape[0]
            s.lut_tmin, s.lut_tmax = 500.0, 30000.0
        if volume is not None:
            dens = np.ascontiguousarray(volume.density, dtype=np.float32)
            self._keep.append(dens)
            s.vol_on = 1
            s.vol = dens.ctypes.data_as(FP)
            s.nr, s.nphi, s.nz = volume.shape
            s.vol_ls_in, s.vol_ls_out, s.vol_zmax = volume.log_s_in, volume.log_s_out, volume.z_max
            s.vol_emis, s.vol_opac, s.vol_stride = volume.emission_scale, volume.opacity_scale, volume.march_stride
            if disc is None:
                lut = np.ascontiguousarray(lut if lut is not None else blackbody_lut(), dtype=np.float32)
                self._keep.append(lut)
                s.bb_lut = lut.ctypes.data_as(FP)
                s.lut_size = lut.shape[0]
                s.lut_tmin, s.lut_tmax = 500.0, 30000.0
        sky = np.ascontiguousarray(sky, dtype=np.float32)
        self._keep.append(sky)
        s.sky = sky.ctypes.data_as(FP)
        s.sky_h, s.sky_w = sky.shape[0], sky.shape[1]
        s.width, s.height = width, height
        if rect is None:
            rect = (0, width, 0, height)
        s.col0, s.cols, s.row0, s.rows = rect
        rpos = float(np.linalg.norm(cam.pos))
        s.semantics, s.integrator = semantics, integrator
        s.dt = dt
        if semantics == SEM_DRAFT:
            re = r_escape if r_escape > 0 else float(np.float32(2.0 * max(rpos, 15.0 * M)))
            if nmax <= 0:
                lg = float(np.log(np.float32(np.float32(re) / np.float32(M))))
                n = math.ceil((75.0 + 6.5 * lg) * float(np.float32(M)) / float(np.float32(dt)))
                nmax = int(min(max(1000, n), 40000))
            s.exit_landing = 0 if exit_landing is None else int(exit_landing)
            s.ju = 0.5 if ju is None else ju
            s.jv = 0.5 if jv is None else jv
        else:
            re = r_escape if r_escape > 0 else max(5.0 * rpos, 100.0)
            s.tspan = tspan if tspan > 0 else max(10.0 * rpos, 500.0)
            nmax = nmax if nmax > 0 else 50000
            s.exit_landing = 1
            s.ju = 1.0 if ju is None else ju
            s.jv = 1.0 if jv is None else jv
        s.r_escape = re
        s.nmax = nmax
        s.hstep_coef, s.hstep_cap = 0.16, 8.0
        s.rtol, s.atol = rtol, atol
        s.tol = tol
        s.relativistic = int(relativistic)
        if starfield is not None:
            self._set_starfield(s, starfield)
        if shutter is not None:
            # (seed, end camera): the end pose's tetrad, as the host computes it
            seed, end = shutter
            u, Ef, Er, Eu = camera_tetrad(end.pos, end.fwd, end.right, end.up_local, M, a,
                                          camera_beta_of(end))
            s.shutter_seed = int(seed)
            s.pos_end[:] = list(map(float, end.pos))
            s.u_end[:], s.Ef_end[:], s.Er_end[:], s.Eu_end[:] = list(u), list(Ef), list(Er), list(Eu)
        self.s = s

    def _set_starfield(self, s, sf):
        """sf: dict of st_starfield's fields (set_starfield! packing,
        src/metal.jl:268-290; star table per _star_lut_cpu, :86-104)."""
        g = np.asarray(sf.get("galactic", (0.0, 0.0, 1.0)), dtype=np.float64)
        gn = float(np.linalg.norm(g))
        n = int(sf.get("table_size", 1024))
        lut = np.ascontiguousarray(star_lut(sf.get("wb_temperature", STAR_WB_TEMPERATURE),
                                            sf.get("saturation", 1.0), n), dtype=np.float32)
        self._keep.append(lut)
        s.star_strength = float(sf.get("strength", 1.0))
        s.star_tw = float(sf.get("texture_weight", 0.0))
        s.star_N = float(sf.get("density", 384.0))
        s.star_fill = float(sf.get("fill", 0.5))
        s.star_sigma = float(sf.get("psf_pixels", 0.5)) * 2.0 * float(sf.get("fov_factor", 0.55)) / int(
            sf.get("height", 1080))
        s.star_flux = float(sf.get("flux", 0.011))
        s.star_g[:] = list(g / gn)
        s.star_conc = float(sf.get("concentration", 3.0))
        s.star_tmin = float(sf.get("temp_min", 3000.0))
        s.star_tspan = float(sf.get("temp_max", 16000.0)) - s.star_tmin
        s.star_lut = lut.ctypes.data_as(FP)
        s.star_lut_size = n
        s.star_seed = int(sf.get("seed", 12345))
        s.star_lut_tmin, s.star_lut_tmax = 500.0, 30000.0

    def trace_dirs(self, dirs, nthreads: int = 0):
        """Per-ray records of rays launched from this scene's camera along
        camera-frame directions dirs[n][3] = (cf, cr, cu) (orc_trace_dirs)."""
        d = np.ascontiguousarray(dirs, dtype=np.float64)
        rays = np.zeros(d.shape[0], dtype=RAY_DTYPE)
        rc = lib().orc_trace_dirs(C.byref(self.s), d.shape[0], d.ctypes.data_as(C.POINTER(C.c_double)),
                                  C.c_void_p(rays.ctypes.data), nthreads)
        if rc != 0:
            raise RuntimeError(f"orc_trace_dirs failed ({rc})")
        return rays

    def render(self, nthreads: int = 0, records: bool = True):
        s = self.s
        out = np.zeros((s.rows, s.cols, 3), dtype=np.float32)
        rays = np.zeros((s.rows, s.cols), dtype=RAY_DTYPE) if records else None
        rc = lib().orc_render(C.byref(s), out.ctypes.data_as(FP),
                              C.c_void_p(rays.ctypes.data) if records else None, nthreads)
        if rc != 0:
            raise RuntimeError(f"orc_render failed ({rc})")
        return out, rays

    def render_depth(self, nb: int, nthreads: int = 0):
        """One unweighted DRAFT pass split into nb depth buckets:
        (rows, cols, nb, 3), the last bucket the sky (orc_render_depth)."""
        s = self.s
        out = np.zeros((s.rows, s.cols, nb, 3), dtype=np.float32)
        rc = lib().orc_render_depth(C.byref(s), int(nb), out.ctypes.data_as(FP), nthreads)
        if rc != 0:
            raise RuntimeError(f"orc_render_depth failed ({rc})")
        return out



def scene_for(w, sky, integrator, width=None, height=None, rect=None, **kw) -> Scene:
    """Oracle scene of a benchmark workload (duck-typed: bh, cam, disc, vol,
    semantics, emitter, params); semantics/emitter codes match the C ABI."""
    disc = None
    if w.disc is not None:
        disc = dict(inner=w.disc.inner_radius, outer=w.disc.outer_radius, falloff=w.disc.density_falloff,
                    wb=w.disc.blackbody.wb_temperature)
    args = dict(cam=w.cam, M=w.bh.M, a=getattr(w.bh, "a", 0.0), sky=sky, width=width or w.width,
                height=height or w.height, semantics=SEM_RENDER if w.semantics == 0 else SEM_DRAFT,
                integrator=integrator, disc=disc, emitter=EMIT_KEPLER if w.emitter == 0 else EMIT_KS_EXACT,
                volume=w.vol, exit_landing=w.params.get("exit_landing"), rect=rect, nmax=w.params.get("nmax", 0))
    args.update(kw)
    return Scene(**args)


# ---- live fluid disc ---------------------------------------------------------

class FluidSim:
    """DiscFluidSim twin (orc_fluid_*): fields are (nphi, nr) float32 arrays,
    the C-order view of the reference's (nr, nphi) column-major matrices."""

    def __init__(self, volume, inner, outer, falloff=0.0, M=1.0, forcing=6.0, drag=0.15, relax=0.05):
        nr, nphi, nz = volume.shape
        self.shape = (nr, nphi, nz)
        self.vu = np.zeros((nphi, nr), np.float32)
        self.vv = np.zeros((nphi, nr), np.float32)
        self.dens = np.zeros((nphi, nr), np.float32)
        self.base = np.zeros((nphi, nr), np.float32)
        self.env = np.zeros((nz, nr), np.float32)
        self.shear = np.zeros(nr, np.float32)
        f = OrcFluid()
        f.nr, f.nphi, f.nz = nr, nphi, nz
        for k in ("vu", "vv", "dens", "base", "env", "shear"):
            setattr(f, k, getattr(self, k).ctypes.data_as(FP))
        f.forcing, f.drag, f.relax = forcing, drag, relax
        self.f = f
        dens = np.ascontiguousarray(volume.density, dtype=np.float32)
        rc = lib().orc_fluid_init(C.byref(f), dens.ctypes.data_as(FP), volume.log_s_in, volume.log_s_out,
                                  volume.z_max, volume.scale_height, M, inner, outer, falloff)
        if rc != 0:
            raise RuntimeError(f"orc_fluid_init failed ({rc})")

    @property
    def t(self) -> float:
        return float(self.f.t)

    def step(self, dt=0.05, jacobi=8, nsteps=1, volume=False):
        """nsteps steps; with volume=True also the extruded (nz, nphi, nr) texture."""
        nr, nphi, nz = self.shape
        vol = np.zeros((nz, nphi, nr), np.float32) if volume else None
        rc = lib().orc_fluid_step(C.byref(self.f), vol.ctypes.data_as(FP) if volume else None, dt, jacobi, nsteps)
        if rc != 0:
            raise RuntimeError(f"orc_fluid_step failed ({rc})")
        return vol
