"""ctypes binding of the test-only host build of the device cut headers."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# RIA_HOSTCHECK_LIB: another build of the same sources (the sanitizer build of `make sanitize`)
LIB = os.environ.get("RIA_HOSTCHECK_LIB") or os.path.join(HERE, "_build", "libhostcheck.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        subprocess.run(["make", "-C", HERE, "-s"], check=True)
        L = ctypes.CDLL(LIB)
        for f in (L.hc_ia_cut, L.hc_mi_cut):
            f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.hc_det_sign.argtypes = [ctypes.c_void_p, ctypes.c_int]
        for f in (L.hc_ia_key2, L.hc_mi_key3, L.hc_ia_key3):
            f.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.hc_sqrt_rn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int]
        _lib = L
    return _lib


def cut(mode, rows, big):
    rows = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1, 4)
    buf = np.zeros(1 << 16, dtype=np.uint8)
    summ = np.zeros(8, dtype=np.uint16)
    f = lib().hc_ia_cut if mode == "ia" else lib().hc_mi_cut
    variant = {"mid": 2, "warp": 3, "warp_light": 4}.get(big, 1 if big is True else 0)
    n = f(rows.shape[0], rows.ctypes.data, variant, buf.ctypes.data, buf.size,
          summ.ctypes.data)
    if n < 0:
        return n, None
    return bytes(buf[:n]), summ.copy()


def det_sign(M):
    M = np.ascontiguousarray(M, dtype=np.float64)
    return lib().hc_det_sign(M.ctypes.data, M.shape[0])


def ia_template(rows):
    """Record of the one-effective-plane path, or None when the tet has two or more planes left."""
    rows = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1, 4)
    L = lib()
    L.hc_ia_template.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    buf = np.zeros(4096, dtype=np.uint8)
    summ = np.zeros(4, dtype=np.uint16)
    n = L.hc_ia_template(rows.shape[0], rows.ctypes.data, buf.ctypes.data, buf.size, summ.ctypes.data)
    assert n not in (-98, -99), "device writer or template summary differs"
    if n < 0:
        return None
    return bytes(buf[:n]), summ.copy()


def ia_template2(rows):
    """Record of the two-group path (the two representatives cut alone, relabelled), or None when the
    tet's planes do not reduce to exactly two groups."""
    rows = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1, 4)
    L = lib()
    L.hc_ia_template2.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    buf = np.zeros(4096, dtype=np.uint8)
    summ = np.zeros(4, dtype=np.uint16)
    n = L.hc_ia_template2(rows.shape[0], rows.ctypes.data, buf.ctypes.data, buf.size, summ.ctypes.data)
    assert n not in (-98, -99), "device writer or template summary differs"
    if n < 0:
        return None
    return bytes(buf[:n]), summ.copy()


def key(mode, rows):
    """Lookup key of two planes (ia), three planes (ia3) or three materials (mi), or None."""
    rows = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1)
    out = np.zeros(1, dtype=np.uint64 if mode == "ia3" else np.uint32)
    f = {"ia": lib().hc_ia_key2, "mi": lib().hc_mi_key3, "ia3": lib().hc_ia_key3}[mode]
    return int(out[0]) if f(rows.ctypes.data, out.ctypes.data) else None


def sqrt_rn(values, perturb=0):
    values = np.ascontiguousarray(values, dtype=np.float64)
    out = np.empty_like(values)
    lib().hc_sqrt_rn(values.ctypes.data, out.ctypes.data, values.size, perturb)
    return out


def div_rn(a, b):
    """The vertex emission's integer-pipe division over two arrays."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    out = np.empty_like(a)
    L = lib()
    L.hc_div_rn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
    L.hc_div_rn(a.ctypes.data, b.ctypes.data, out.ctypes.data, a.size)
    return out


def robust(mode, rows, forge=0):
    """The device's robust-test outcome of one tet (0 ok, 1 counts differ, 2 the given order fails, 3 the
    reversed order fails); forge 1..3 plants that outcome in the cut wrapper of the harness."""
    rows = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1, 4)
    L = lib()
    L.hc_robust.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    return L.hc_robust(1 if mode == "mi" else 0, rows.shape[0], rows.ctypes.data, forge)
