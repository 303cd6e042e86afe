"""Python mirror of the reference's pipeline entry points over the C ABI (tests and benchmark).

  implicit_arrangement(pts, tets, func_vals, ...)   src/implicit_arrangement.h:39-62
  material_interface(pts, tets, func_vals, ...)     src/material_interface.h:38-61
  grid_implicit_arrangement / grid_material_interface: tet5 grid + sampling on the device
  compute_arrangement_batch / compute_material_interface_batch: the per-tet
      simplicial_arrangement calls for many tets at once
Results come back as numpy arrays; every computation runs on the GPU.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .functions import FUNC_DTYPE


class Mesh:
    """Owner of a ria_mesh handle (device buffers); fields are copied to the host on demand."""

    _FIELDS = {
        "xyz": (_lib.FIELD_POINTS, np.float64, (-1, 3)),
        "verts": (_lib.FIELD_VERTS, np.int64, (-1, 11)),
        "face_offsets": (_lib.FIELD_FACE_OFFSETS, np.int64, None),
        "face_verts": (_lib.FIELD_FACE_VERTS, np.int64, None),
        "face_tet_offsets": (_lib.FIELD_FACE_TET_OFFSETS, np.int64, None),
        "face_tets": (_lib.FIELD_FACE_TETS, np.int64, (-1, 2)),
        "face_func": (_lib.FIELD_FACE_FUNC, np.int64, (-1, 2)),
        "func_in_tet": (_lib.FIELD_FUNC_IN_TET, np.int64, None),
        "start_index": (_lib.FIELD_START_INDEX, np.int64, None),
        "rec_offsets": (_lib.FIELD_REC_OFFSETS, np.int64, None),
        "rec_bytes": (_lib.FIELD_REC_BYTES, np.uint8, None),
        "func_vals": (_lib.FIELD_FUNC_VALS, np.float64, None),
        # local-to-global maps (the reference's extraction variants for useTopoRayShooting = false)
        "tet_vert_offsets": (_lib.FIELD_TET_VERT_OFFSETS, np.int64, None),
        "tet_verts": (_lib.FIELD_TET_VERTS, np.int64, None),
        "tet_face_offsets": (_lib.FIELD_TET_FACE_OFFSETS, np.int64, None),
        "tet_faces": (_lib.FIELD_TET_FACES, np.int64, None),
        # mesh connectivity (compute_mesh_edges / compute_patches / compute_chains)
        "edges": (_lib.FIELD_EDGES, np.int64, (-1, 2)),
        "edge_face_offsets": (_lib.FIELD_EDGE_FACE_OFFSETS, np.int64, None),
        "edge_faces": (_lib.FIELD_EDGE_FACES, np.int64, (-1, 2)),
        "face_edges": (_lib.FIELD_FACE_EDGES, np.int64, None),
        "patch_offsets": (_lib.FIELD_PATCH_OFFSETS, np.int64, None),
        "patch_faces": (_lib.FIELD_PATCH_FACES, np.int64, None),
        "patch_label": (_lib.FIELD_PATCH_LABELS, np.int64, (-1, 2)),
        "chain_offsets": (_lib.FIELD_CHAIN_OFFSETS, np.int64, None),
        "chain_edges": (_lib.FIELD_CHAIN_EDGES, np.int64, None),
    }

    def __init__(self, handle):
        self._h = handle
        self._cache = {}

    def __del__(self):
        self.close()

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().ria_mesh_free(self._h)
            self._h = None

    def _copy(self, field, dtype):
        L = _lib.load()
        n = int(L.ria_mesh_count(self._h, field))
        out = np.zeros(max(n, 1), dtype=dtype)
        # copied even when empty: a field built on first request reports its error here
        _lib.check(L.ria_mesh_copy(self._h, field, out.ctypes.data))
        return out[:n]

    def copy_into(self, name, out):
        """Copy a field into a caller buffer (e.g. pinned host memory); returns the filled view."""
        field, dt, shape = self._FIELDS[name]
        L = _lib.load()
        n = int(L.ria_mesh_count(self._h, field))
        flat = out.reshape(-1).view(dt)
        if flat.size < n:
            raise ValueError("buffer too small for %s: %d < %d" % (name, flat.size, n))
        if n:
            _lib.check(L.ria_mesh_copy(self._h, field, flat.ctypes.data))
        v = flat[:n]
        return v.reshape(shape) if shape else v

    def __getitem__(self, name):
        if name not in self._cache:
            if name == "stats":
                a = np.zeros(len(_lib.STAT_NAMES), dtype=np.int64)
                _lib.check(_lib.load().ria_mesh_copy(self._h, _lib.FIELD_STATS, a.ctypes.data))
                self._cache[name] = a
            elif name == "timings":
                a = np.zeros(len(_lib.TIMING_NAMES), dtype=np.float64)
                _lib.check(_lib.load().ria_mesh_copy(self._h, _lib.FIELD_TIMINGS, a.ctypes.data))
                self._cache[name] = a
            else:
                field, dt, shape = self._FIELDS[name]
                a = self._copy(field, dt)
                self._cache[name] = a.reshape(shape) if shape else a
        return self._cache[name]

    @property
    def stats(self) -> dict:
        return dict(zip(_lib.STAT_NAMES, self["stats"].tolist()))

    @property
    def timings(self) -> dict:
        return dict(zip(_lib.TIMING_NAMES, self["timings"].tolist()))

    def csg(self, tree=None, positive_inside=True) -> np.ndarray:
        """Per-face CSG label (0 not on the boundary, 1 inside on the positive side, 2 on the negative
        side); tree: list of (op, a, b) units as the reference's CSG tree files, None = union."""
        t, n = _csg_tree(tree)
        out = np.zeros(int(_lib.load().ria_mesh_count(self._h, _lib.FIELD_FACE_FUNC)) // 2, dtype=np.uint8)
        _lib.check(_lib.load().ria_mesh_csg(self._h, t.ctypes.data if n else None, n, int(positive_inside),
                                            out.ctypes.data))
        return out


    def face_sides(self) -> np.ndarray:
        """n_faces x 2 sign vectors (bit j: function j positive) on the positive / negative side."""
        n = int(_lib.load().ria_mesh_count(self._h, _lib.FIELD_FACE_FUNC)) // 2
        out = np.zeros((n, 2), dtype=np.uint64)
        _lib.check(_lib.load().ria_mesh_face_sides(self._h, out.ctypes.data))
        return out


CSG_OPS = {"Intersection": 0, "Union": 1, "Negation": 2}


def _csg_tree(tree):
    if not tree:
        return np.zeros(3, dtype=np.int32), 0
    rows = []
    for u in tree:
        if isinstance(u, dict):
            rows.append((CSG_OPS[u["type"]], int(u["elements"][0]), int(u["elements"][1])))
        else:
            rows.append(tuple(int(x) for x in u))
    return np.ascontiguousarray(rows, dtype=np.int32), len(rows)


def _config(use_lookup=True, use_secondary_lookup=True, use_topo_ray_shooting=True, robust_test=False):
    if not use_lookup:
        use_secondary_lookup = False
    return _lib.Config(int(use_lookup), int(use_secondary_lookup), int(use_topo_ray_shooting), int(robust_test), 1)


def _run_host(name, pts, tets, func_vals, **kw):
    L = _lib.load()
    pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
    tets = np.ascontiguousarray(tets, dtype=np.int64).reshape(-1, 4)
    fv = np.ascontiguousarray(func_vals, dtype=np.float64)
    if fv.ndim != 2 or fv.shape[0] != pts.shape[0]:
        raise ValueError("func_vals must be n_pts x n_func")
    cfg = _config(**kw)
    h = ctypes.c_void_p()
    st = getattr(L, name)(ctypes.byref(cfg), pts.ctypes.data, pts.shape[0], tets.ctypes.data, tets.shape[0],
                          fv.ctypes.data, fv.shape[1], ctypes.byref(h))
    return _mesh_or_raise(st, h, kw)


def implicit_arrangement(pts, tets, func_vals, **kw) -> Mesh:
    return _run_host("ria_compute_implicit_arrangement", pts, tets, func_vals, **kw)


def material_interface(pts, tets, func_vals, **kw) -> Mesh:
    return _run_host("ria_compute_material_interface", pts, tets, func_vals, **kw)


def _run_grid(name, res, funcs, bbox_min=(-1.0, -1.0, -1.0), bbox_max=(1.0, 1.0, 1.0), **kw):
    L = _lib.load()
    funcs = np.ascontiguousarray(funcs, dtype=FUNC_DTYPE)
    bmin = np.asarray(bbox_min, dtype=np.float64)
    bmax = np.asarray(bbox_max, dtype=np.float64)
    cfg = _config(**kw)
    h = ctypes.c_void_p()
    st = getattr(L, name)(ctypes.byref(cfg), int(res), bmin.ctypes.data, bmax.ctypes.data, funcs.ctypes.data,
                          len(funcs), ctypes.byref(h))
    return _mesh_or_raise(st, h, kw)


def _mesh_or_raise(st, h, kw):
    """The mesh of a call; a robust test whose tets failed (RIA_EINTERNAL with a mesh) still returns
    it, since its statistics count the failing tets of each type."""
    if st == _lib.RIA_EINTERNAL and kw.get("robust_test") and h.value:
        return Mesh(h)
    _lib.check(st)
    return Mesh(h)


def grid_implicit_arrangement(res, funcs, **kw) -> Mesh:
    return _run_grid("ria_grid_implicit_arrangement", res, funcs, **kw)


def grid_material_interface(res, funcs, **kw) -> Mesh:
    return _run_grid("ria_grid_material_interface", res, funcs, **kw)


class BatchMesh(Mesh):
    """A ria_grid_batch result; `problem(i)` views one problem's fields, numbered as in its own grid
    call."""

    def __len__(self):
        return int(_lib.load().ria_batch_size(self._h))

    def problem(self, i):
        return _ProblemView(self, int(i))


class _ProblemView:
    def __init__(self, batch, i):
        self._b = batch
        self._i = i
        self._cache = {}

    def __getitem__(self, name):
        if name not in self._cache:
            L = _lib.load()
            h = self._b._h
            if name == "stats":
                a = np.zeros(len(_lib.STAT_NAMES), dtype=np.int64)
                _lib.check(L.ria_batch_copy(h, self._i, _lib.FIELD_STATS, a.ctypes.data))
            elif name == "timings":
                a = np.zeros(len(_lib.TIMING_NAMES), dtype=np.float64)
                _lib.check(L.ria_batch_copy(h, self._i, _lib.FIELD_TIMINGS, a.ctypes.data))
            else:
                field, dt, shape = Mesh._FIELDS[name]
                n = int(L.ria_batch_count(h, self._i, field))
                a = np.zeros(n, dtype=dt)
                if n:
                    _lib.check(L.ria_batch_copy(h, self._i, field, a.ctypes.data))
                if shape:
                    a = a.reshape(shape)
            self._cache[name] = a
        return self._cache[name]

    @property
    def stats(self) -> dict:
        return dict(zip(_lib.STAT_NAMES, self["stats"].tolist()))

    def csg(self, tree=None, positive_inside=True) -> np.ndarray:
        t, n = _csg_tree(tree)
        out = np.zeros(len(self["face_func"]), dtype=np.uint8)
        _lib.check(_lib.load().ria_batch_csg(self._b._h, self._i, t.ctypes.data if n else None, n,
                                             int(positive_inside), out.ctypes.data))
        return out


def _problem_array(problems):
    """ria_grid_problem array of (res, funcs[, bbox_min, bbox_max]) tuples, and the arrays it points to."""
    arr = (_lib.GridProblem * len(problems))()
    keep = []
    for i, pr in enumerate(problems):
        res, funcs = pr[0], np.ascontiguousarray(pr[1], dtype=FUNC_DTYPE)
        bmin = pr[2] if len(pr) > 2 else (-1.0, -1.0, -1.0)
        bmax = pr[3] if len(pr) > 3 else (1.0, 1.0, 1.0)
        keep.append(funcs)
        arr[i].resolution = int(res)
        arr[i].n_func = len(funcs)
        for a in range(3):
            arr[i].bbox_min[a] = float(bmin[a])
            arr[i].bbox_max[a] = float(bmax[a])
        arr[i].funcs = funcs.ctypes.data
    return arr, keep


def grid_batch(problems, mode="ia", **kw) -> BatchMesh:
    """Solve many grid problems in one pass of every stage.  problems: iterable of
    (res, funcs) or (res, funcs, bbox_min, bbox_max)."""
    L = _lib.load()
    problems = list(problems)
    arr, keep = _problem_array(problems)
    cfg = _config(**kw)
    h = ctypes.c_void_p()
    _lib.check(L.ria_grid_batch(ctypes.byref(cfg), 1 if mode == "mi" else 0, arr, len(problems), ctypes.byref(h)))
    return BatchMesh(h)


_TUNING_KEYS = ("warp_route", "warp_blocks_per_sm", "fast_block", "mid_threshold", "cut_graph", "heavy_min_k",
                "mi_heavy_min_k")


def get_tuning() -> dict:
    """The current device's tuning record of the per-tet cut (ria_tuning)."""
    t = _lib.Tuning()
    _lib.check(_lib.load().ria_get_tuning(ctypes.byref(t)))
    return {k: getattr(t, k) for k in _TUNING_KEYS}


def set_tuning(tuning: dict) -> None:
    t = _lib.Tuning(*[int(tuning[k]) for k in _TUNING_KEYS])
    _lib.check(_lib.load().ria_set_tuning(ctypes.byref(t)))


def autotune(problems, mode="ia", reps=2, **kw):
    """The project's autotuner (ria_autotune) on a sample of batched problems: installs the fastest
    tuning record on the current device; returns (record, its median seconds, the previous record's)."""
    problems = list(problems)
    arr, keep = _problem_array(problems)
    cfg = _config(**kw)
    t = _lib.Tuning()
    best, dflt = ctypes.c_double(), ctypes.c_double()
    _lib.check(_lib.load().ria_autotune(ctypes.byref(cfg), 1 if mode == "mi" else 0, arr, len(problems), int(reps),
                                        ctypes.byref(t), ctypes.byref(best), ctypes.byref(dflt)))
    return {k: getattr(t, k) for k in _TUNING_KEYS}, best.value, dflt.value


class _Borrowed:
    """A mesh handle owned by the server (not freed here)."""

    def __init__(self, h):
        self._h = h


class Server:
    """The served form (ria_server_*): submit requests as they arrive, wait for their results."""

    KINDS = {"ia": _lib.REQ_IA, "mi": _lib.REQ_MI, "csg": _lib.REQ_CSG}

    def __init__(self, budget_bytes, streams=3, max_batch=256, **kw):
        cfg = _config(**kw)
        self._h = ctypes.c_void_p()
        _lib.check(_lib.load().ria_server_create(ctypes.byref(cfg), int(budget_bytes), int(streams), int(max_batch),
                                                 ctypes.byref(self._h)))
        self._keep = {}

    def submit(self, kind, res, funcs, bbox_min=(-1.0, -1.0, -1.0), bbox_max=(1.0, 1.0, 1.0), tree=None,
               positive_inside=True) -> int:
        funcs = np.ascontiguousarray(funcs, dtype=FUNC_DTYPE)
        t, n = _csg_tree(tree)
        q = _lib.Request()
        q.kind = self.KINDS[kind]
        q.grid.resolution = int(res)
        q.grid.n_func = len(funcs)
        for a in range(3):
            q.grid.bbox_min[a] = float(bbox_min[a])
            q.grid.bbox_max[a] = float(bbox_max[a])
        q.grid.funcs = funcs.ctypes.data
        q.csg_tree = t.ctypes.data if n else None
        q.csg_units = n
        q.positive_inside = int(positive_inside)
        ticket = ctypes.c_uint64()
        _lib.check(_lib.load().ria_server_submit(self._h, ctypes.byref(q), ctypes.byref(ticket)))
        return int(ticket.value)

    def wait(self, ticket, timeout=-1.0):
        """(view of the result, latency in seconds); the view reads like a grid call's mesh."""
        h, prob, lat = ctypes.c_void_p(), ctypes.c_uint32(), ctypes.c_double()
        _lib.check(_lib.load().ria_server_wait(self._h, int(ticket), float(timeout), ctypes.byref(h),
                                               ctypes.byref(prob), ctypes.byref(lat)))
        return _ProblemView(_Borrowed(h), prob.value), lat.value

    def labels(self, ticket) -> np.ndarray:
        L = _lib.load()
        n = int(L.ria_server_labels(self._h, int(ticket), None))
        out = np.zeros(n, dtype=np.uint8)
        if n:
            L.ria_server_labels(self._h, int(ticket), out.ctypes.data)
        return out

    def release(self, ticket):
        _lib.load().ria_server_release(self._h, int(ticket))

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().ria_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def sample_functions(funcs, pts, out=None) -> np.ndarray:
    L = _lib.load()
    funcs = np.ascontiguousarray(funcs, dtype=FUNC_DTYPE)
    pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
    if out is None:
        out = np.zeros((pts.shape[0], len(funcs)))
    elif out.dtype != np.float64 or out.shape != (pts.shape[0], len(funcs)) or not out.flags.c_contiguous:
        raise ValueError("out must be a contiguous n_pts x n_func float64 array")
    _lib.check(L.ria_sample_functions(funcs.ctypes.data, len(funcs), pts.ctypes.data, pts.shape[0], out.ctypes.data))
    return out


def _batch(name, rows_per_tet):
    L = _lib.load()
    offs = np.zeros(len(rows_per_tet) + 1, dtype=np.uint32)
    for i, r in enumerate(rows_per_tet):
        offs[i + 1] = offs[i] + len(r)
    vals = np.ascontiguousarray(np.concatenate([np.asarray(r, dtype=np.float64).reshape(-1, 4) for r in rows_per_tet])
                                if len(rows_per_tet) else np.zeros((0, 4)))
    cap = 6144 * max(1, len(rows_per_tet))
    buf = np.zeros(cap, dtype=np.uint8)
    roff = np.zeros(len(rows_per_tet) + 1, dtype=np.uint64)
    _lib.check(getattr(L, name)(vals.ctypes.data, offs.ctypes.data, len(rows_per_tet), buf.ctypes.data, cap,
                                roff.ctypes.data))
    return [bytes(buf[int(roff[i]):int(roff[i + 1])]) for i in range(len(rows_per_tet))]


def compute_arrangement_batch(planes_per_tet) -> list[bytes]:
    """Canonical arrangement record of each tet (rows: 4 corner values per plane)."""
    return _batch("ria_compute_arrangement_batch", planes_per_tet)


def compute_material_interface_batch(materials_per_tet) -> list[bytes]:
    return _batch("ria_compute_material_interface_batch", materials_per_tet)


def device_count() -> int:
    return int(_lib.load().ria_device_count())
