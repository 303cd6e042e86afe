"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module; the
product path never does.  `build()` compiles oracle/_build/libria_oracle.so with the Makefile
beside this file.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# RIA_ORACLE_LIB: another build of the same sources (the sanitizer build of `make sanitize`)
LIB_PATH = os.environ.get("RIA_ORACLE_LIB") or os.path.join(HERE, "_build", "libria_oracle.so")

_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-C", HERE, "-s"], check=True)
    else:
        subprocess.run(["make", "-C", HERE, "-s"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.oracle_ia_cut.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.oracle_mi_cut.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.oracle_grid.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_sample.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int]
        L.oracle_run.restype = ctypes.c_void_p
        L.oracle_run.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                 ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_len.restype = ctypes.c_int64
        L.oracle_len.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        L.oracle_copy.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
        L.oracle_free.argtypes = [ctypes.c_void_p]
        L.oracle_set_selfcheck.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def set_selfcheck(on: bool):
    lib().oracle_set_selfcheck(1 if on else 0)


def ia_cut(planes) -> bytes:
    p = np.ascontiguousarray(planes, dtype=np.float64).reshape(-1, 4)
    buf = np.zeros(1 << 20, dtype=np.uint8)
    n = lib().oracle_ia_cut(p.shape[0], p.ctypes.data, buf.ctypes.data, buf.size)
    if n < 0:
        raise RuntimeError(f"oracle ia_cut failed ({n})")
    return bytes(buf[:n])


def mi_cut(materials) -> bytes:
    p = np.ascontiguousarray(materials, dtype=np.float64).reshape(-1, 4)
    buf = np.zeros(1 << 20, dtype=np.uint8)
    n = lib().oracle_mi_cut(p.shape[0], p.ctypes.data, buf.ctypes.data, buf.size)
    if n < 0:
        raise RuntimeError(f"oracle mi_cut failed ({n})")
    return bytes(buf[:n])


def grid(res: int, bmin=(-1.0, -1.0, -1.0), bmax=(1.0, 1.0, 1.0)):
    n = res + 1
    pts = np.zeros((n ** 3, 3))
    tets = np.zeros((5 * res ** 3, 4), dtype=np.int64)
    bmn = np.asarray(bmin, dtype=np.float64)
    bmx = np.asarray(bmax, dtype=np.float64)
    lib().oracle_grid(res, bmn.ctypes.data, bmx.ctypes.data, pts.ctypes.data, tets.ctypes.data)
    return pts, tets


def sample(funcs, pts, threads=1):
    funcs = np.ascontiguousarray(funcs)
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    out = np.zeros((pts.shape[0], len(funcs)))
    lib().oracle_sample(funcs.ctypes.data, len(funcs), pts.ctypes.data, pts.shape[0], out.ctypes.data, threads)
    return out


_ARRAYS = {
    "func_in_tet": np.int64, "start_index": np.int64, "rec_offsets": np.int64, "rec_bytes": np.uint8,
    "verts": np.int64, "xyz": np.float64, "face_offsets": np.int64, "face_verts": np.int64,
    "face_tet_offsets": np.int64, "face_tets": np.int64, "face_func": np.int64, "edges": np.int64,
    "patch_offsets": np.int64, "patch_faces": np.int64, "patch_label": np.int64, "chain_offsets": np.int64,
    "chain_edges": np.int64, "nm_degree": np.int64, "stats": np.int64, "timings": np.float64,
    "edge_face_offsets": np.int64, "edge_faces": np.int64, "face_edges": np.int64,
    "tet_vert_offsets": np.int64, "tet_verts": np.int64, "tet_face_offsets": np.int64, "tet_faces": np.int64,
}

STAT_NAMES = ["num_pts", "num_tets", "num_degenerate_vertex", "num_intersecting_tet", "num_a_func",
              "num_b_func", "num_more_func", "num_verts", "num_faces", "num_exact_predicates"]


def run(mode: str, pts, tets, func_vals, threads: int = 1, connectivity: bool = False) -> dict:
    """Run stages (b)-(d) (plus optional edges/patches/chains) on the CPU; returns numpy arrays."""
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    tets = np.ascontiguousarray(tets, dtype=np.int64)
    fv = np.ascontiguousarray(func_vals, dtype=np.float64)
    L = lib()
    h = L.oracle_run(0 if mode == "ia" else 1, pts.ctypes.data, pts.shape[0], tets.ctypes.data, tets.shape[0],
                     fv.ctypes.data, fv.shape[1], threads, 1 if connectivity else 0)
    out = {}
    try:
        for name, dt in _ARRAYS.items():
            n = L.oracle_len(h, name.encode())
            a = np.zeros(n, dtype=dt)
            if n:
                L.oracle_copy(h, name.encode(), a.ctypes.data)
            out[name] = a
    finally:
        L.oracle_free(h)
    out["verts"] = out["verts"].reshape(-1, 11)
    out["xyz"] = out["xyz"].reshape(-1, 3)
    out["face_tets"] = out["face_tets"].reshape(-1, 2)
    out["face_func"] = out["face_func"].reshape(-1, 2)
    out["edges"] = out["edges"].reshape(-1, 2)
    out["patch_label"] = out["patch_label"].reshape(-1, 2)
    out["stats_named"] = dict(zip(STAT_NAMES, out["stats"].tolist()))
    return out
