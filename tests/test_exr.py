"""Uncompressed OpenEXR files without the OpenEXR library: the AOV writer
round-trips through the env-map reader, which returns what readExr's
Imf::RgbaInputFile gives (half-precision RGBA, missing alpha 1); a file with
HALF channels written here byte by byte reads back exactly."""
import ctypes as C
import struct

import numpy as np

from lightgraph_gb300 import _capi


def write(path, w, h, planes: dict):
    lib = _capi.load_host()
    names = (C.c_char_p * len(planes))(*[k.encode() for k in planes])
    arrs = [np.ascontiguousarray(v, np.float32) for v in planes.values()]
    ptrs = (C.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
    assert lib.lg_write_exr(str(path).encode(), w, h, len(arrs), names, ptrs) == 0


def read(path):
    lib = _capi.load_host()
    w, h = C.c_int32(), C.c_int32()
    assert lib.lg_read_exr_rgba(str(path).encode(), C.byref(w), C.byref(h), None) == 0
    out = np.zeros((h.value, w.value, 4), np.float32)
    assert lib.lg_read_exr_rgba(str(path).encode(), C.byref(w), C.byref(h), _capi.ptr(out)) == 0
    return out


def test_float_roundtrip_is_half_rounded(tmp_path):
    rng = np.random.default_rng(3)
    w, h = 7, 5
    R, G, B = (rng.random((h, w)) * 100.0 - 20.0).astype(np.float32), rng.random((h, w)).astype(np.float32), \
        (rng.random((h, w)) * 1e-5).astype(np.float32)
    write(tmp_path / "a.exr", w, h, {"R": R, "G": G, "B": B, "direct.R": R})
    img = read(tmp_path / "a.exr")
    for c, v in enumerate((R, G, B)):
        assert np.array_equal(img[..., c], v.astype(np.float16).astype(np.float32))
    assert np.all(img[..., 3] == 1.0)


def test_half_channels_read_exactly(tmp_path):
    w, h = 3, 2
    vals = np.array([[0.5, -2.0, 32000.0], [6.1e-5, 1e-7, 0.0]], np.float16)
    hdr = struct.pack("<ii", 20000630, 2)

    def attr(name, typ, val):
        return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(val)) + val
    chl = b"".join(n + b"\0" + struct.pack("<i", 1) + b"\0\0\0\0" + struct.pack("<ii", 1, 1) for n in (b"G", b"R"))
    chl += b"\0"
    box = struct.pack("<iiii", 10, 20, 10 + w - 1, 20 + h - 1)
    hdr += attr("channels", "chlist", chl) + attr("compression", "compression", b"\0")
    hdr += attr("dataWindow", "box2i", box) + attr("displayWindow", "box2i", box)
    hdr += attr("lineOrder", "lineOrder", b"\0") + b"\0"
    rows = []
    for y in range(h):
        data = vals[y].tobytes() + (vals[y] * 2).astype(np.float16).tobytes()  # G then R
        rows.append(struct.pack("<ii", 20 + y, len(data)) + data)
    off = len(hdr) + 8 * h
    table = b""
    for r in rows:
        table += struct.pack("<Q", off)
        off += len(r)
    (tmp_path / "h.exr").write_bytes(hdr + table + b"".join(rows))
    img = read(tmp_path / "h.exr")
    assert img.shape == (h, w, 4)
    assert np.array_equal(img[..., 1], vals.astype(np.float32))
    assert np.array_equal(img[..., 0], (vals * 2).astype(np.float16).astype(np.float32))
    assert np.all(img[..., 2] == 0.0) and np.all(img[..., 3] == 1.0)
