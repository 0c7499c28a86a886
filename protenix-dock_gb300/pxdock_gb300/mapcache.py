"""The reference's receptor-map cache files (receptor_cache::save / restore,
engine/src/core/grid.cpp:305-431) through the library's host-side codec
(pxd_bdg_* / pxd_meta_*): a <tag>.bdg Boost binary archive per map holding its
{E, dE/dx, dE/dy, dE/dz} records, and the meta.dat Boost text archive with the format
version 20241030, the box and the excluded receptor atoms. No device is touched.

`ReusableEngine.dump_maps` / `load_maps` write and read these files; the functions here
convert them for other tools (e.g. a map built by the reference's `bdgen`).
"""
import ctypes as C

import numpy as np

from . import abi, native

FORMAT_VERSION = 20241030


def _lib():
    return native.load()


def _check(n):
    if n < 0:
        raise native.NativeError(-n, "map cache codec: %s" % ("malformed input" if -n == 4 else "invalid argument"))
    return n


def encode_bdg(records, value_bytes=8):
    """records (P, 4) -> the bytes of a <tag>.bdg archive (param_t double: 8, float: 4)."""
    rec = np.ascontiguousarray(records, dtype=np.float64).reshape(-1, 4)
    lib = _lib()
    p = rec.ctypes.data_as(abi.f64p)
    n = _check(lib.pxd_bdg_encode(p, rec.shape[0], value_bytes, None, 0))
    buf = C.create_string_buffer(n)
    _check(lib.pxd_bdg_encode(p, rec.shape[0], value_bytes, buf, n))
    return buf.raw[:n]


def decode_bdg(data):
    """bytes of a .bdg archive -> ((P, 4) float64 records, value_bytes)."""
    lib = _lib()
    vb = C.c_int32(0)
    n = _check(lib.pxd_bdg_decode(data, len(data), None, 0, C.byref(vb)))
    out = np.empty((n, 4), dtype=np.float64)
    _check(lib.pxd_bdg_decode(data, len(data), out.ctypes.data_as(abi.f64p), n, C.byref(vb)))
    return out, vb.value


def encode_meta(init_xyz, npoints, spacing, excluded=()):
    """The meta.dat text of a box (origin, points per axis, spacing) and excluded atoms."""
    box = abi.Box()
    box.init_xyz[:] = [float(v) for v in init_xyz]
    box.npoints[:] = [int(v) for v in npoints]
    box.spacing = float(spacing)
    ex = np.ascontiguousarray(list(excluded), dtype=np.int64)
    exp = ex.ctypes.data_as(C.POINTER(C.c_int64))
    lib = _lib()
    n = _check(lib.pxd_meta_encode(C.byref(box), exp, ex.size, None, 0))
    buf = C.create_string_buffer(n + 1)
    _check(lib.pxd_meta_encode(C.byref(box), exp, ex.size, buf, n + 1))
    return buf.value.decode()


def decode_meta(text):
    """meta.dat text -> dict(version, init_xyz, npoints, spacing, excluded); only
    version is set when it is not FORMAT_VERSION."""
    raw = text.encode() if isinstance(text, str) else bytes(text)
    lib = _lib()
    box, ver = abi.Box(), C.c_uint64(0)
    n = _check(lib.pxd_meta_decode(raw, len(raw), C.byref(box), C.byref(ver), None, 0))
    ex = np.empty(n, dtype=np.int64)
    _check(lib.pxd_meta_decode(raw, len(raw), C.byref(box), C.byref(ver), ex.ctypes.data_as(C.POINTER(C.c_int64)), n))
    return dict(version=ver.value, init_xyz=list(box.init_xyz), npoints=list(box.npoints), spacing=box.spacing,
                excluded=ex.tolist())
