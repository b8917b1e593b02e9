"""ctypes declarations of the C ABI in include/spacetime_gb300.h.

The structs below mirror the header field for field; `load()` opens the
in-tree libspacetime_gb300.so and raises if it is missing (there is no CPU
fallback for the render path).
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("SPACETIME_GB300_LIB", os.path.join(_HERE, "libspacetime_gb300.so"))

ST_OK, ST_EINVAL, ST_ECUDA, ST_EBUDGET, ST_ENOMEM, ST_EUNSUPPORTED, ST_ESTATE, ST_ELIMIT = range(8)
ST_PROJ_PINHOLE, ST_PROJ_FISHEYE = 0, 1
ST_EMIT_KEPLER, ST_EMIT_KS_EXACT = 0, 1
ST_SEM_RENDER, ST_SEM_DRAFT = 0, 1
ST_PREC_FP64, ST_PREC_FP32_GUARDED, ST_PREC_FP32, ST_PREC_FP32_GUARDED_DF = 0, 1, 2, 3
ST_SCHED_PIXEL, ST_SCHED_PERSISTENT = 0, 1

ST_RAY_ESCAPED = 1
ST_RAY_CAPTURED = 2
ST_RAY_BUDGET = 4
ST_RAY_BLACK = 8
ST_RAY_CROSSED = 16
ST_RAY_GRAZE = 32
ST_RAY_BCAPT = 64
ST_RAY_SURROGATE = 128
ST_RAY_GUARDED = 256

D3 = C.c_double * 3


class StCamera(C.Structure):
    _fields_ = [
        ("pos", D3), ("fwd", D3), ("right", D3), ("up", D3),
        ("fov_factor", C.c_double), ("velocity", D3),
        ("projection", C.c_int), ("fisheye_deg", C.c_double),
        ("aperture_world", C.c_double), ("focus_dist", C.c_double),
    ]


class StSpacetime(C.Structure):
    _fields_ = [("M", C.c_double), ("a", C.c_double)]


class StDisc(C.Structure):
    _fields_ = [
        ("inner", C.c_double), ("outer", C.c_double), ("falloff", C.c_double),
        ("wb_temperature", C.c_double), ("table_min", C.c_double), ("table_max", C.c_double),
        ("table_size", C.c_int), ("emitter", C.c_int),
    ]


class StFluidParams(C.Structure):
    _fields_ = [("M", C.c_double), ("forcing", C.c_double), ("drag", C.c_double), ("relax", C.c_double),
                ("scale_height", C.c_double)]


class StVolume(C.Structure):
    _fields_ = [
        ("density", C.POINTER(C.c_float)), ("nr", C.c_int), ("nphi", C.c_int), ("nz", C.c_int),
        ("log_s_in", C.c_float), ("log_s_out", C.c_float), ("z_max", C.c_float),
        ("emission_scale", C.c_float), ("opacity_scale", C.c_float), ("march_stride", C.c_int),
    ]


class StStarfield(C.Structure):
    _fields_ = [
        ("strength", C.c_double), ("texture_weight", C.c_double), ("height", C.c_int),
        ("fov_factor", C.c_double), ("density", C.c_double), ("fill", C.c_double), ("flux", C.c_double),
        ("psf_pixels", C.c_double), ("galactic", C.c_double * 3), ("concentration", C.c_double),
        ("temp_min", C.c_double), ("temp_max", C.c_double), ("seed", C.c_int),
        ("wb_temperature", C.c_double), ("saturation", C.c_double), ("table_size", C.c_int),
    ]


class StRenderParams(C.Structure):
    _fields_ = [
        ("width", C.c_int), ("height", C.c_int), ("samples", C.c_int),
        ("dt", C.c_double), ("nmax", C.c_int),
        ("semantics", C.c_int), ("precision", C.c_int), ("schedule", C.c_int),
        ("r_escape", C.c_double), ("tspan", C.c_double),
        ("relativistic", C.c_int), ("exit_landing", C.c_int), ("pixel_jitter", C.c_int),
        ("seed", C.c_ulonglong),
        ("r_guard", C.c_double), ("crit_band", C.c_double), ("crit_r", C.c_double), ("renorm_every", C.c_int),
        ("surrogate", C.c_int), ("surrogate_sigma", C.c_double),
        ("block_x", C.c_int), ("block_y", C.c_int), ("chunk_steps", C.c_int), ("graph", C.c_int),
        ("order", C.c_int), ("tol", C.c_double),
        ("refine", C.c_int), ("refine_var", C.c_double), ("refine_graze", C.c_double), ("refine_margin", C.c_int),
    ]


class StStats(C.Structure):
    _fields_ = [
        ("total_ms", C.c_double), ("kernel_ms", C.c_double),
        ("rays", C.c_ulonglong), ("steps", C.c_ulonglong), ("fp64_steps", C.c_ulonglong),
        ("gas_samples", C.c_ulonglong), ("surrogate_rays", C.c_ulonglong),
        ("launches", C.c_int), ("status", C.c_int),
        ("h2d_bytes", C.c_ulonglong), ("d2h_bytes", C.c_ulonglong),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class StRayDiag(C.Structure):
    _fields_ = [
        ("dir", C.c_double * 3), ("r_final", C.c_float), ("alpha", C.c_float), ("r_cross", C.c_float),
        ("g_cross", C.c_float), ("lambda_", C.c_float), ("flags", C.c_int), ("steps", C.c_int),
        ("fp64_steps", C.c_int), ("pad", C.c_int * 2),
    ]


# numpy view of st_ray_diag records
DIAG_DTYPE = [
    ("dir", "<f8", (3,)), ("r_final", "<f4"), ("alpha", "<f4"), ("r_cross", "<f4"), ("g_cross", "<f4"),
    ("lambda_", "<f4"), ("flags", "<i4"), ("steps", "<i4"), ("fp64_steps", "<i4"), ("pad", "<i4", (2,)),
]

# Every symbol include/spacetime_gb300.h declares.
EXPORTS = [
    "st_abi_version", "st_strerror", "st_render_params_default",
    "st_context_create", "st_context_set_disc", "st_context_set_volume", "st_context_destroy",
    "st_render", "st_render_diag", "st_render_device", "st_render_frames", "st_camera_tetrad",
    "st_surrogate_create", "st_surrogate_destroy", "st_surrogate_num_params", "st_surrogate_get_params",
    "st_surrogate_set_params", "st_surrogate_forward", "st_surrogate_forward_tc", "st_surrogate_loss_grad", "st_surrogate_generate",
    "st_surrogate_train", "st_render_frames_noalloc", "st_context_set_surrogate",
    "st_starfield_default", "st_context_set_starfield", "st_render_motion",
    "st_save_raw", "st_load_raw_size", "st_load_raw", "st_sky_fan", "st_render_layered",
    "st_render_depth", "st_render_layered_ring", "st_fluid_params_default", "st_fluid_create", "st_fluid_step", "st_fluid_state",
    "st_fluid_destroy", "st_measure_fp32_peak",
]
ST_FAN_N, ST_FAN_FINE = 4096, 1024

_lib = None


class StError(RuntimeError):
    def __init__(self, code: int, where: str):
        msg = _lib.st_strerror(code).decode() if _lib is not None else str(code)
        super().__init__(f"{where}: {msg} (status {code})")
        self.code = code


def load(path: str | None = None) -> C.CDLL:
    """Open libspacetime_gb300.so (built by spacetime_gb300.build)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
        )
    lib = C.CDLL(p)
    P = C.POINTER
    lib.st_abi_version.restype = C.c_int
    lib.st_strerror.restype = C.c_char_p
    lib.st_strerror.argtypes = [C.c_int]
    lib.st_render_params_default.argtypes = [P(StRenderParams), C.c_int]
    lib.st_context_create.argtypes = [P(C.c_void_p), P(C.c_float), C.c_int, C.c_int, C.c_int]
    lib.st_context_set_disc.argtypes = [C.c_void_p, P(StDisc)]
    lib.st_context_set_volume.argtypes = [C.c_void_p, P(StVolume)]
    lib.st_context_destroy.argtypes = [C.c_void_p]
    lib.st_context_destroy.restype = None
    lib.st_render.argtypes = [C.c_void_p, P(StCamera), P(StSpacetime), P(StRenderParams),
                              P(C.c_float), P(StStats)]
    lib.st_render_diag.argtypes = [C.c_void_p, P(StCamera), P(StSpacetime), P(StRenderParams),
                                   P(C.c_float), C.c_void_p, P(StStats)]
    lib.st_render_device.argtypes = [C.c_void_p, P(StCamera), P(StSpacetime), P(StRenderParams),
                                     P(C.c_void_p), P(StStats)]
    lib.st_render_frames.argtypes = [C.c_void_p, C.c_int, P(StCamera), P(StSpacetime),
                                     P(StRenderParams), P(C.c_float), P(StStats)]
    lib.st_camera_tetrad.argtypes = [P(StCamera), P(StSpacetime), P(C.c_double)]
    FP, LL = P(C.c_float), C.c_longlong
    lib.st_surrogate_create.argtypes = [P(C.c_void_p), C.c_int, C.c_ulonglong]
    lib.st_surrogate_destroy.argtypes = [C.c_void_p]
    lib.st_surrogate_destroy.restype = None
    lib.st_surrogate_num_params.argtypes = []
    lib.st_surrogate_get_params.argtypes = [C.c_void_p, FP]
    lib.st_surrogate_set_params.argtypes = [C.c_void_p, FP]
    lib.st_surrogate_forward.argtypes = [C.c_void_p, FP, C.c_int, FP]
    lib.st_surrogate_forward_tc.argtypes = [C.c_void_p, FP, C.c_int, FP]
    lib.st_surrogate_loss_grad.argtypes = [C.c_void_p, FP, FP, C.c_int, FP, FP]
    lib.st_surrogate_generate.argtypes = [C.c_void_p, LL, LL, C.c_double, FP, FP, FP]
    lib.st_surrogate_train.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float, FP]
    lib.st_render_frames_noalloc.argtypes = [C.c_void_p, C.c_int, C.c_int, P(StDisc), C.c_void_p, P(StVolume),
                                             C.c_int, P(StCamera), P(StSpacetime), P(StRenderParams), C.c_void_p,
                                             C.c_void_p, P(StStats)]
    lib.st_render_frames_noalloc.restype = C.c_int
    lib.st_context_set_surrogate.argtypes = [C.c_void_p, C.c_void_p]
    lib.st_context_set_surrogate.restype = C.c_int
    lib.st_starfield_default.argtypes = [P(StStarfield)]
    lib.st_starfield_default.restype = None
    lib.st_context_set_starfield.argtypes = [C.c_void_p, P(StStarfield)]
    lib.st_context_set_starfield.restype = C.c_int
    lib.st_render_motion.argtypes = [C.c_void_p, P(StCamera), P(StCamera), C.c_int, C.c_int, P(StSpacetime),
                                     P(StRenderParams), P(C.c_float), C.c_void_p, P(StStats)]
    lib.st_render_motion.restype = C.c_int
    lib.st_save_raw.argtypes = [C.c_char_p, P(C.c_float), C.c_int, C.c_int, C.c_char_p]
    lib.st_save_raw.restype = C.c_int
    lib.st_load_raw_size.argtypes = [C.c_char_p, P(C.c_int), P(C.c_int)]
    lib.st_load_raw_size.restype = C.c_int
    lib.st_load_raw.argtypes = [C.c_char_p, P(C.c_float), C.c_int, C.c_int]
    lib.st_load_raw.restype = C.c_int
    lib.st_sky_fan.argtypes = [C.c_void_p, P(StCamera), P(StSpacetime), P(StRenderParams), P(C.c_float),
                               P(C.c_float), P(C.c_float)]
    lib.st_sky_fan.restype = C.c_int
    lib.st_render_layered.argtypes = [C.c_void_p, P(StCamera), P(StSpacetime), P(StRenderParams), C.c_int, C.c_int,
                                      P(C.c_float), C.c_void_p, P(StStats)]
    lib.st_render_layered.restype = C.c_int
    lib.st_render_layered_ring.argtypes = [C.c_void_p, P(StCamera), P(StSpacetime), P(StRenderParams), C.c_int,
                                           C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, P(C.c_float),
                                           C.c_void_p, P(StStats)]
    lib.st_render_layered_ring.restype = C.c_int
    lib.st_render_depth.argtypes = [C.c_void_p, P(StCamera), P(StSpacetime), P(StRenderParams), C.c_int,
                                    P(C.c_float), P(StStats)]
    lib.st_render_depth.restype = C.c_int
    lib.st_fluid_params_default.argtypes = [P(StFluidParams)]
    lib.st_fluid_params_default.restype = None
    lib.st_fluid_create.argtypes = [P(C.c_void_p), C.c_void_p, P(StDisc), P(StFluidParams)]
    lib.st_fluid_create.restype = C.c_int
    lib.st_fluid_step.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int, P(C.c_float)]
    lib.st_fluid_step.restype = C.c_int
    lib.st_fluid_state.argtypes = [C.c_void_p, P(C.c_float), P(C.c_float), P(C.c_float), P(C.c_float),
                                   P(C.c_double)]
    lib.st_fluid_state.restype = C.c_int
    lib.st_measure_fp32_peak.argtypes = [C.c_int, C.c_int, P(C.c_double), P(C.c_double)]
    lib.st_measure_fp32_peak.restype = C.c_int
    lib.st_fluid_destroy.argtypes = [C.c_void_p]
    lib.st_fluid_destroy.restype = None
    for name in ("st_context_create", "st_context_set_disc", "st_context_set_volume", "st_render",
                 "st_render_diag", "st_render_device", "st_render_frames", "st_camera_tetrad",
                 "st_surrogate_create", "st_surrogate_num_params", "st_surrogate_get_params",
                 "st_surrogate_set_params", "st_surrogate_forward", "st_surrogate_forward_tc", "st_surrogate_loss_grad",
                 "st_surrogate_generate", "st_surrogate_train"):
        getattr(lib, name).restype = C.c_int
    if path is None:
        _lib = lib
    return lib


def check(code: int, where: str) -> None:
    if code != ST_OK:
        raise StError(code, where)
