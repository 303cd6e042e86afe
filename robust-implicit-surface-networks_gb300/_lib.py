"""ctypes binding of the C ABI (include/ria.h) for the Python test and benchmark harnesses.

The library is built in-tree by build.py.  Loading fails loudly if it is missing: there is no
Python or CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libria.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "ria.h")

RIA_OK, RIA_EINVAL, RIA_ENOMEM, RIA_ECAPACITY, RIA_EDEGENERATE, RIA_ETIMEOUT, RIA_ECUDA, RIA_EINTERNAL, RIA_ENODEVICE = range(9)

(FIELD_POINTS, FIELD_VERTS, FIELD_FACE_OFFSETS, FIELD_FACE_VERTS, FIELD_FACE_TET_OFFSETS, FIELD_FACE_TETS,
 FIELD_FACE_FUNC, FIELD_FUNC_IN_TET, FIELD_START_INDEX, FIELD_REC_OFFSETS, FIELD_REC_BYTES, FIELD_STATS,
 FIELD_TIMINGS, FIELD_FUNC_VALS, FIELD_TET_VERT_OFFSETS, FIELD_TET_VERTS, FIELD_TET_FACE_OFFSETS,
 FIELD_TET_FACES, FIELD_EDGES, FIELD_EDGE_FACE_OFFSETS, FIELD_EDGE_FACES, FIELD_FACE_EDGES, FIELD_PATCH_OFFSETS,
 FIELD_PATCH_FACES, FIELD_PATCH_LABELS, FIELD_CHAIN_OFFSETS, FIELD_CHAIN_EDGES) = range(27)

STAT_NAMES = ["num_pts", "num_tets", "num_degenerate_vertex", "num_intersecting_tet", "num_a_func", "num_b_func",
              "num_more_func", "num_verts", "num_faces", "num_deferred", "robust_failures", "robust_type2",
              "robust_type3"]
TIMING_NAMES = ["sample", "filter", "cut", "extract", "total"]


class RiaError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"ria status {status}: {msg}")
        self.status = status


class GridProblem(ctypes.Structure):
    """ria_grid_problem of include/ria.h."""
    _fields_ = [("resolution", ctypes.c_uint32), ("n_func", ctypes.c_uint32), ("bbox_min", ctypes.c_double * 3),
                ("bbox_max", ctypes.c_double * 3), ("funcs", ctypes.c_void_p)]


class Request(ctypes.Structure):
    """ria_request of include/ria.h."""
    _fields_ = [("kind", ctypes.c_int32), ("grid", GridProblem), ("csg_tree", ctypes.c_void_p),
                ("csg_units", ctypes.c_uint32), ("positive_inside", ctypes.c_int32)]


REQ_IA, REQ_MI, REQ_CSG = 0, 1, 2


class Tuning(ctypes.Structure):
    """ria_tuning of include/ria.h."""
    _fields_ = [("warp_route", ctypes.c_int64), ("warp_blocks_per_sm", ctypes.c_int32), ("fast_block", ctypes.c_int32),
                ("mid_threshold", ctypes.c_int64), ("cut_graph", ctypes.c_int32), ("heavy_min_k", ctypes.c_int32),
                ("mi_heavy_min_k", ctypes.c_int32)]


class Config(ctypes.Structure):
    _fields_ = [("use_lookup", ctypes.c_int32), ("use_secondary_lookup", ctypes.c_int32),
                ("use_topo_ray_shooting", ctypes.c_int32), ("robust_test", ctypes.c_int32),
                ("keep_records", ctypes.c_int32)]


def declared_functions() -> list[str]:
    """Names of every function declared in include/ria.h."""
    with open(HEADER) as f:
        src = f.read()
    return re.findall(r"RIA_API\s+[\w\s\*]+?\b(ria_\w+)\s*\(", src)


_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with build.py (there is no fallback path)")
    L = ctypes.CDLL(LIB_PATH)
    vp, u64, u32, i32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int32
    cfgp = ctypes.POINTER(Config)
    for name in ("ria_compute_implicit_arrangement", "ria_compute_material_interface"):
        fn = getattr(L, name)
        fn.restype = i32
        fn.argtypes = [cfgp, vp, u64, vp, u64, vp, u32, ctypes.POINTER(vp)]
    for name in ("ria_compute_implicit_arrangement_device", "ria_compute_material_interface_device"):
        fn = getattr(L, name)
        fn.restype = i32
        fn.argtypes = [cfgp, vp, u64, vp, u64, vp, u32, vp, ctypes.POINTER(vp)]
    for name in ("ria_grid_implicit_arrangement", "ria_grid_material_interface"):
        fn = getattr(L, name)
        fn.restype = i32
        fn.argtypes = [cfgp, u32, vp, vp, vp, u32, ctypes.POINTER(vp)]
    L.ria_sample_functions.restype = i32
    L.ria_sample_functions.argtypes = [vp, u32, vp, u64, vp]
    for name in ("ria_compute_arrangement_batch", "ria_compute_material_interface_batch"):
        fn = getattr(L, name)
        fn.restype = i32
        fn.argtypes = [vp, vp, u64, vp, u64, vp]
    L.ria_compute_arrangement_batch_noalloc.restype = i32
    L.ria_compute_arrangement_batch_noalloc.argtypes = [vp, vp, u64, vp, u64, vp, vp]
    L.ria_grid_batch.restype = i32
    L.ria_grid_batch.argtypes = [cfgp, i32, vp, u32, ctypes.POINTER(vp)]
    L.ria_batch_size.restype = u32
    L.ria_batch_size.argtypes = [vp]
    L.ria_batch_count.restype = u64
    L.ria_batch_count.argtypes = [vp, u32, i32]
    L.ria_batch_copy.restype = i32
    L.ria_batch_copy.argtypes = [vp, u32, i32, vp]
    L.ria_mesh_csg.restype = i32
    L.ria_mesh_csg.argtypes = [vp, vp, u32, i32, vp]
    L.ria_mesh_face_sides.restype = i32
    L.ria_mesh_face_sides.argtypes = [vp, vp]
    L.ria_batch_csg.restype = i32
    L.ria_batch_csg.argtypes = [vp, u32, vp, u32, i32, vp]
    L.ria_server_create.restype = i32
    L.ria_server_create.argtypes = [cfgp, u64, u32, u32, ctypes.POINTER(vp)]
    L.ria_server_submit.restype = i32
    L.ria_server_submit.argtypes = [vp, ctypes.POINTER(Request), ctypes.POINTER(u64)]
    L.ria_server_wait.restype = i32
    L.ria_server_wait.argtypes = [vp, u64, ctypes.c_double, ctypes.POINTER(vp), ctypes.POINTER(u32),
                                  ctypes.POINTER(ctypes.c_double)]
    L.ria_server_labels.restype = u64
    L.ria_server_labels.argtypes = [vp, u64, vp]
    L.ria_server_release.restype = None
    L.ria_server_release.argtypes = [vp, u64]
    L.ria_server_destroy.restype = None
    L.ria_server_destroy.argtypes = [vp]
    L.ria_mesh_count.restype = u64
    L.ria_mesh_count.argtypes = [vp, i32]
    L.ria_mesh_copy.restype = i32
    L.ria_mesh_copy.argtypes = [vp, i32, vp]
    L.ria_mesh_free.restype = None
    L.ria_mesh_free.argtypes = [vp]
    L.ria_last_error.restype = ctypes.c_char_p
    L.ria_last_error.argtypes = []
    L.ria_device_count.restype = ctypes.c_int
    L.ria_device_count.argtypes = []
    L.ria_lookup_cache_clear.restype = i32
    L.ria_lookup_cache_clear.argtypes = []
    L.ria_get_tuning.restype = i32
    L.ria_get_tuning.argtypes = [ctypes.POINTER(Tuning)]
    L.ria_set_tuning.restype = i32
    L.ria_set_tuning.argtypes = [ctypes.POINTER(Tuning)]
    L.ria_autotune.restype = i32
    L.ria_autotune.argtypes = [cfgp, i32, vp, u32, u32, ctypes.POINTER(Tuning), ctypes.POINTER(ctypes.c_double),
                               ctypes.POINTER(ctypes.c_double)]
    L.ria_measure_fp64_rate.restype = i32
    L.ria_measure_fp64_rate.argtypes = [i32, ctypes.POINTER(ctypes.c_double)]
    L.ria_kernel_launches.restype = u64
    L.ria_kernel_launches.argtypes = []
    _lib = L
    return L


def check(status: int):
    if status != RIA_OK:
        raise RiaError(status, load().ria_last_error().decode())
