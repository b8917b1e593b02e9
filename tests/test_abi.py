"""The C ABI without a GPU: the library loads, exports every function the
header declares, its struct layouts match the ctypes mirror, and the host-only
entry points behave (defaults, error strings, argument checks)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from spacetime_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "spacetime_gb300.h")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(st_\w+)\s*\(", text, flags=re.M)))


def test_header_and_mirror_list_agree():
    assert header_functions() == sorted(_abi.EXPORTS)


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(built_lib)
    for name in header_functions():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\sT\s(st_\w+)", out))
    assert set(header_functions()) <= exported


def test_abi_version_and_strerror(built_lib):
    lib = _abi.load()
    ver = int(re.search(r"#define ST_ABI_VERSION (\d+)", open(HEADER).read()).group(1))
    assert lib.st_abi_version() == ver
    for code in range(8):
        assert lib.st_strerror(code)
    assert lib.st_strerror(99) == b"unknown status"


_PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include "spacetime_gb300.h"
#define S(T) printf(#T " %zu\n", sizeof(T));
#define O(T, f) printf(#T "." #f " %zu\n", offsetof(T, f));
int main(void) {
  S(st_camera) S(st_spacetime) S(st_disc) S(st_volume) S(st_render_params) S(st_stats) S(st_ray_diag)
  O(st_camera, focus_dist) O(st_camera, projection) O(st_disc, emitter) O(st_volume, march_stride)
  O(st_render_params, seed) O(st_render_params, chunk_steps) O(st_render_params, surrogate_sigma)
  O(st_stats, d2h_bytes) O(st_ray_diag, flags) O(st_ray_diag, fp64_steps)
  O(st_render_params, graph) O(st_render_params, order) O(st_render_params, tol)
  O(st_render_params, refine) O(st_render_params, refine_var) O(st_render_params, refine_margin)
  S(st_starfield) O(st_starfield, table_size) O(st_starfield, seed) O(st_starfield, galactic)
  return 0;
}
"""


def test_struct_layouts_match_ctypes(tmp_path):
    src = tmp_path / "probe.c"
    src.write_text(_PROBE)
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split("\n")
               if line)
    mirror = {"st_camera": _abi.StCamera, "st_spacetime": _abi.StSpacetime, "st_disc": _abi.StDisc,
              "st_volume": _abi.StVolume, "st_render_params": _abi.StRenderParams, "st_stats": _abi.StStats,
              "st_ray_diag": _abi.StRayDiag, "st_starfield": _abi.StStarfield}
    for name, cls in mirror.items():
        assert int(got[name]) == C.sizeof(cls), name
    for key, val in got.items():
        if "." in key:
            t, f = key.split(".")
            fname = "lambda_" if f == "lambda" else f
            assert getattr(mirror[t], fname).offset == int(val), key
    assert np.dtype(_abi.DIAG_DTYPE).itemsize == C.sizeof(_abi.StRayDiag)


def test_params_default_match_reference_keywords(built_lib):
    lib = _abi.load()
    p = _abi.StRenderParams()
    lib.st_render_params_default(C.byref(p), _abi.ST_SEM_RENDER)
    # render(...; width=400, height=200, samples=1), src/raytrace.jl:339-350
    assert (p.width, p.height, p.samples, p.precision) == (400, 200, 1, _abi.ST_PREC_FP64)
    assert p.exit_landing == 1
    lib.st_render_params_default(C.byref(p), _abi.ST_SEM_DRAFT)
    # render_draft_mtl(...; width=1920, height=1080, samples=2, dt=0.02), src/metal.jl:2040-2054
    assert (p.width, p.height, p.samples, p.dt) == (1920, 1080, 2, 0.02)
    assert p.precision == _abi.ST_PREC_FP32 and p.pixel_jitter == 1


def _gpu_present():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_argument_errors_without_gpu(built_lib):
    lib = _abi.load()
    h = C.c_void_p()
    sky = np.zeros((4, 8, 3), np.float32)
    fp = sky.ctypes.data_as(C.POINTER(C.c_float))
    assert lib.st_context_create(None, fp, 8, 4, 0) == _abi.ST_EINVAL
    assert lib.st_context_create(C.byref(h), None, 8, 4, 0) == _abi.ST_EINVAL
    assert lib.st_context_create(C.byref(h), fp, 1, 4, 0) == _abi.ST_EINVAL
    assert lib.st_context_set_disc(None, None) == _abi.ST_EINVAL
    assert lib.st_render(None, None, None, None, None, None) == _abi.ST_EINVAL
    cam = _abi.StCamera()
    assert lib.st_camera_tetrad(C.byref(cam), C.byref(_abi.StSpacetime(1.0, 1.5)),
                                (C.c_double * 16)()) == _abi.ST_EINVAL
    if not _gpu_present():
        assert lib.st_context_create(C.byref(h), fp, 8, 4, 0) == _abi.ST_ECUDA


def test_host_tetrad_matches_oracle(built_lib, oracle_lib):
    """st_camera_tetrad is host FP64 code: check it against the oracle."""
    from spacetime_gb300 import api, scene
    for pos, a, vel in [((0, -30, 3), 0.0, (0, 0, 0)), ((14.8, 0, 2.6), 0.9, (0, 0.3, 0)),
                        ((2.3, 0.4, 0.1), 0.0, (0.1, 0.2, 0)), ((1.9, 0.2, 0.5), 0.99, (0, 0, 0))]:
        cam = scene.Camera.look_at(pos, (0, 0, 0), (0, 0, 1.0), 0.75, velocity=vel)
        bh = api.Kerr(1.0, a) if a else api.Schwarzschild(1.0)
        T = api.camera_tetrad(cam, bh)
        beta = scene.camera_beta(cam)
        ref = oracle_lib.camera_tetrad(cam.pos, cam.fwd, cam.right, cam.up_local, 1.0, a, beta)
        assert np.abs(T - np.stack(ref)).max() < 1e-13


def test_surrogate_row_widths_match_header():
    """The Python handle sizes label rows as the header documents them."""
    from spacetime_gb300 import surrogate
    hdr = open(os.path.join(os.path.dirname(__file__), "..", "include", "spacetime_gb300.h")).read()
    assert f"raw[n][{surrogate.RAW}]" in hdr
    assert f"t[n][{surrogate.NT}]" in hdr
    assert f"out[n][{surrogate.NOUT}]" in hdr and f"x[n][{surrogate.NIN}]" in hdr


def _julia_fields(src, name):
    m = re.search(r"struct " + name + r"\n(.*?)\n(?:    " + name + r"\(\) = new\(\)\n)?end", src, re.S)
    assert m, name
    body = re.sub(r"#.*", "", m.group(1))
    return [f.split("::")[0].strip() for f in re.split(r"[;\n]", body) if "::" in f]


def test_julia_binding_structs_follow_the_c_layout():
    """The Julia module's ccall structs list the C structs' fields in order."""
    src = open(os.path.join(os.path.dirname(__file__), "..", "julia", "SpaceTimeGB300.jl")).read()
    for jname, cstruct in (("StRenderParams", _abi.StRenderParams), ("StStarfield", _abi.StStarfield),
                           ("StCamera", _abi.StCamera), ("StDisc", _abi.StDisc), ("StVolume", _abi.StVolume),
                           ("StFluidParams", _abi.StFluidParams)):
        assert _julia_fields(src, jname) == [f for f, _ in cstruct._fields_], jname
