"""Raw HDR frame files: save_raw / load_raw (src/rawio.jl:18-42) over the C ABI
(st_save_raw / st_load_raw, host only).

A frame is the renderer's (height, width, 3) float32 array (row 0 = v < 0).
The file is a linear, unclamped 32-bit float RGB TIFF in display orientation
-- the reference's rotr90 of its (width, height) matrix, which for this array
is a left-right flip -- and a TOML sidecar <path>.toml with the metadata plus
`format` and `saved_at`.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

from . import _abi

FORMAT = "SpaceTime raw v1: linear Float32 RGB, display orientation"


def _toml_value(v) -> str:
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    if isinstance(v, (float, np.floating)):
        f = float(v)
        if math.isnan(f):
            return "nan"
        if math.isinf(f):
            return "inf" if f > 0 else "-inf"
        return repr(f)
    if isinstance(v, str):
        return '"' + v.replace("\\", "\\\\").replace('"', '\\"').replace("\n", "\\n") + '"'
    if isinstance(v, (list, tuple, np.ndarray)):
        return "[" + ", ".join(_toml_value(x) for x in v) + "]"
    raise TypeError(f"metadata value {v!r} is not TOML-representable (numbers, strings, booleans, vectors)")


def to_toml(meta: dict) -> str:
    """Flat TOML text of `meta` (keys sorted, as TOML.print writes a Dict)."""
    lines = []
    for k in sorted(meta):
        if k in ("format", "saved_at"):
            continue
        lines.append(f"{k} = {_toml_value(meta[k])}")
    return "\n".join(lines) + ("\n" if lines else "")


def save_raw(path: str, img: np.ndarray, metadata: dict | None = None) -> str:
    img = np.ascontiguousarray(img, dtype=np.float32)
    if img.ndim != 3 or img.shape[2] != 3:
        raise ValueError("img must be (height, width, 3)")
    h, w, _ = img.shape
    text = to_toml(metadata or {}).encode()
    lib = _abi.load()
    _abi.check(lib.st_save_raw(os.fsencode(path), img.ctypes.data_as(C.POINTER(C.c_float)), w, h, text or None),
               "st_save_raw")
    return path


def load_raw(path: str) -> tuple[np.ndarray, dict]:
    lib = _abi.load()
    w, h = C.c_int(), C.c_int()
    _abi.check(lib.st_load_raw_size(os.fsencode(path), C.byref(w), C.byref(h)), "st_load_raw_size")
    img = np.empty((h.value, w.value, 3), dtype=np.float32)
    _abi.check(lib.st_load_raw(os.fsencode(path), img.ctypes.data_as(C.POINTER(C.c_float)), w.value, h.value),
               "st_load_raw")
    side = path + ".toml"
    meta = {}
    if os.path.isfile(side):
        import tomllib
        with open(side, "rb") as f:
            meta = tomllib.load(f)
    return img, meta
