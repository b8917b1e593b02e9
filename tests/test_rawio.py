"""Raw HDR frame files (save_raw / load_raw, src/rawio.jl:18-42), host side:
bit-exact round trip of unclamped float32 frames, the display orientation
(the reference's rotr90), the sidecar, and a TIFF readable as a standard
32-bit float RGB image."""
import struct

import numpy as np
import pytest

from spacetime_gb300 import rawio


@pytest.fixture
def frame():
    rng = np.random.default_rng(7)
    img = rng.lognormal(-3, 2, (27, 48, 3)).astype(np.float32)   # HDR, unclamped
    img[0, 0] = [np.inf, -0.0, 1e-38]
    img[5, 7] = [65504.0, 3.4e38, 0.0]
    return img


def test_round_trip_is_bit_exact(built_lib, tmp_path, frame):
    p = str(tmp_path / "f.tif")
    rawio.save_raw(p, frame, {"width": 48, "height": 27, "camera": "config0", "fov": 0.75,
                              "pos": [0.0, -30.0, 3.0], "relativistic": False})
    back, meta = rawio.load_raw(p)
    assert back.dtype == np.float32 and back.shape == frame.shape
    assert np.array_equal(back.view(np.uint32), frame.view(np.uint32))
    assert meta["format"] == rawio.FORMAT and "saved_at" in meta
    assert meta["pos"] == [0.0, -30.0, 3.0] and meta["camera"] == "config0" and meta["relativistic"] is False


def _read_tiff(path):
    """Minimal independent reader of the one-strip little-endian file."""
    d = open(path, "rb").read()
    assert d[:4] == b"II*\x00"
    ifd = struct.unpack_from("<I", d, 4)[0]
    n = struct.unpack_from("<H", d, ifd)[0]
    tags = {}
    for e in range(n):
        t, typ, cnt, val = struct.unpack_from("<HHII", d, ifd + 2 + 12 * e)
        if typ == 3 and cnt == 1:
            val &= 0xFFFF
        tags[t] = (typ, cnt, val)
    w, h = tags[256][2], tags[257][2]
    assert tags[259][2] == 1 and tags[262][2] == 2 and tags[277][2] == 3 and tags[284][2] == 1
    bps = struct.unpack_from("<3H", d, tags[258][2])
    fmt = struct.unpack_from("<3H", d, tags[339][2])
    assert bps == (32, 32, 32) and fmt == (3, 3, 3)
    off = tags[273][2]
    return np.frombuffer(d, dtype="<f4", count=w * h * 3, offset=off).reshape(h, w, 3)


def test_display_orientation_is_rotr90(built_lib, tmp_path, frame):
    p = str(tmp_path / "o.tif")
    rawio.save_raw(p, frame)
    tif = _read_tiff(p)
    # rotr90 of the (width, height) matrix: TIFF (row r, col c) = frame pixel (width-1-c, r)
    assert np.array_equal(tif.view(np.uint32), frame[:, ::-1].view(np.uint32))


def test_metadata_must_be_toml_representable(built_lib, tmp_path, frame):
    with pytest.raises(TypeError):
        rawio.save_raw(str(tmp_path / "x.tif"), frame, {"bad": object()})


def test_rejects_a_size_mismatch(built_lib, tmp_path, frame):
    import ctypes as C
    from spacetime_gb300 import _abi
    p = str(tmp_path / "s.tif")
    rawio.save_raw(p, frame)
    buf = np.empty(10 * 10 * 3, np.float32)
    rc = _abi.load().st_load_raw(p.encode(), buf.ctypes.data_as(C.POINTER(C.c_float)), 10, 10)
    assert rc == _abi.ST_EINVAL
