"""Implicit function descriptors, tet grids and the synthetic workloads.

The reference samples its functions through the absent `implicit_functions` library
(called at app/implicit_arrangement.cpp:59, app/material_interface.cpp:62, app/csg.cpp:184) and
reads them from JSON lists such as examples/tests/2-planesphere.json.  This module parses that
JSON format into `ria_function` records (layout and formulas in include/ria.h) and builds the
seeded synthetic workloads used by the tests and the benchmark.

Supported types and sign conventions (distance-like primitives are positive inside):
  plane    {point, normal}                  n . (x - p)
  sphere   {center, radius, squared?}       r - |x - c|      (squared: r^2 - |x - c|^2)
  cylinder {axis_point, axis_vector, radius} r - dist(x, axis)
  torus    {center, axis_vector, major_radius, minor_radius}
                                            r - dist(x, core circle)
  zero                                      0
Every type honours "is_flipped" (negation).  The positive-inside sphere convention is the one
under which the oracle reproduces the reference's material-interface known answers
(tests/test_implicit_networks.cpp:601-640 and :685-731, patch label order).  line, circle, cone,
rbf and shader are not supported (ValueError).
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass, field

import numpy as np

FUNC_ZERO, FUNC_PLANE, FUNC_SPHERE, FUNC_SPHERE_SQ, FUNC_CYLINDER, FUNC_TORUS = range(6)

# matches `ria_function` in include/ria.h
FUNC_DTYPE = np.dtype([("type", "<i4"), ("flipped", "<i4"), ("p", "<f8", (12,))])


def _unit(v):
    # fixed evaluation order (x*x + y*y) + z*z, rounded after each operation, as the C++ loader
    v = np.asarray(v, dtype=np.float64)
    n = float(np.sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]))
    if n == 0.0:
        raise ValueError("zero axis vector")
    return v / n


def make_functions(specs: list[dict]) -> np.ndarray:
    """Pack a list of reference-style JSON function objects into a ria_function array."""
    out = np.zeros(len(specs), dtype=FUNC_DTYPE)
    for i, s in enumerate(specs):
        t = s["type"]
        p = np.zeros(12)
        if t == "zero":
            ty = FUNC_ZERO
        elif t == "plane":
            ty = FUNC_PLANE
            p[0:3] = s["point"]
            p[3:6] = s["normal"]
        elif t == "sphere":
            ty = FUNC_SPHERE_SQ if s.get("squared", False) else FUNC_SPHERE
            p[0:3] = s["center"]
            p[3] = s["radius"]
        elif t == "cylinder":
            ty = FUNC_CYLINDER
            p[0:3] = s["axis_point"]
            p[3:6] = _unit(s["axis_vector"])
            p[6] = s["radius"]
        elif t == "torus":
            ty = FUNC_TORUS
            p[0:3] = s["center"]
            p[3:6] = _unit(s["axis_vector"])
            p[6] = s["major_radius"]
            p[7] = s["minor_radius"]
        else:
            raise ValueError(f"unsupported implicit function type {t!r}")
        out[i]["type"] = ty
        out[i]["flipped"] = 1 if s.get("is_flipped", False) else 0
        out[i]["p"] = p
    return out


def load_functions(path: str) -> np.ndarray:
    with open(path) as f:
        return make_functions(json.load(f))


def grid_coords(res: int, bmin=(-1.0, -1.0, -1.0), bmax=(1.0, 1.0, 1.0)):
    """Per-axis grid coordinates, rounded exactly as src/io.cpp:104-106 computes them."""
    n = res + 1
    t = np.arange(n, dtype=np.float64) / np.float64(n - 1)
    return [t * (np.float64(bmax[a]) - np.float64(bmin[a])) + np.float64(bmin[a]) for a in range(3)]


def generate_tet_mesh(res: int, bmin=(-1.0, -1.0, -1.0), bmax=(1.0, 1.0, 1.0)):
    """tet5 grid of src/io.cpp:95-152: vertex i*N*N + j*N + k, five tets per cube."""
    n = res + 1
    xs, ys, zs = grid_coords(res, bmin, bmax)
    pts = np.empty((n, n, n, 3))
    pts[..., 0] = xs[:, None, None]
    pts[..., 1] = ys[None, :, None]
    pts[..., 2] = zs[None, None, :]
    pts = pts.reshape(-1, 3)
    i, j, k = np.meshgrid(np.arange(res), np.arange(res), np.arange(res), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    v0 = i * n * n + j * n + k
    v1 = (i + 1) * n * n + j * n + k
    v2 = (i + 1) * n * n + (j + 1) * n + k
    v3 = i * n * n + (j + 1) * n + k
    v4, v5, v6, v7 = v0 + 1, v1 + 1, v2 + 1, v3 + 1
    even = ((i + j + k) % 2) == 0
    a = np.stack([
        np.stack([v4, v6, v1, v3], 1), np.stack([v6, v3, v4, v7], 1), np.stack([v1, v3, v0, v4], 1),
        np.stack([v3, v1, v2, v6], 1), np.stack([v4, v1, v6, v5], 1)], 1)
    b = np.stack([
        np.stack([v7, v0, v2, v5], 1), np.stack([v2, v3, v0, v7], 1), np.stack([v5, v7, v0, v4], 1),
        np.stack([v7, v2, v6, v5], 1), np.stack([v0, v1, v2, v5], 1)], 1)
    tets = np.where(even[:, None, None], a, b).reshape(-1, 4).astype(np.int64)
    return pts, tets


def load_tet_mesh(path: str):
    """Tet mesh JSON of src/io.cpp:65-93: [[pts...], [tets...]]."""
    with open(path) as f:
        data = json.load(f)
    return np.asarray(data[0], dtype=np.float64).reshape(-1, 3), np.asarray(data[1], dtype=np.int64).reshape(-1, 4)


# ---------------------------------------------------------------------------------------------
# configuration files (src/io.cpp:19-63)

@dataclass
class Config:
    tet_mesh_file: str = ""
    tet_mesh_resolution: int = 0
    tet_mesh_bbox_min: tuple = (-1.0, -1.0, -1.0)
    tet_mesh_bbox_max: tuple = (1.0, 1.0, 1.0)
    func_file: str = ""
    output_dir: str = ""
    use_lookup: bool = True
    use_secondary_lookup: bool = True
    use_topo_ray_shooting: bool = True


def parse_config_file(path: str) -> Config:
    """Parse a reference JSON config.  Relative paths resolve against the config's folder.

    Unlike src/io.cpp:59-61, missing lookup switches default to true (as the reference README
    documents).
    """
    if not os.path.exists(path):
        raise RuntimeError("Config file does not exist!")
    with open(path) as f:
        data = json.load(f)
    base = os.path.dirname(os.path.abspath(path))

    def resolve(p):
        return p if os.path.isabs(p) else os.path.abspath(os.path.join(base, p))

    c = Config()
    if "tetMeshFile" in data:
        c.tet_mesh_file = resolve(data["tetMeshFile"])
    else:
        c.tet_mesh_resolution = int(data["gridResolution"])
        c.tet_mesh_bbox_min = tuple(float(x) for x in data["gridBbox"][0])
        c.tet_mesh_bbox_max = tuple(float(x) for x in data["gridBbox"][1])
    c.func_file = resolve(data["funcFile"])
    c.output_dir = resolve(data.get("outputDir", "."))
    c.use_lookup = bool(data.get("useLookup", True))
    c.use_secondary_lookup = bool(data.get("useSecondaryLookup", True))
    c.use_topo_ray_shooting = bool(data.get("useTopoRayShooting", True))
    return c


# ---------------------------------------------------------------------------------------------
# seeded synthetic workloads

@dataclass
class Workload:
    name: str
    mode: str          # "ia" or "mi"
    res: int           # cubes per axis
    funcs: np.ndarray  # ria_function records
    bbox_min: tuple = (-1.0, -1.0, -1.0)
    bbox_max: tuple = (1.0, 1.0, 1.0)
    use_lookup: bool = True
    use_secondary_lookup: bool = True
    meta: dict = field(default_factory=dict)

    @property
    def n_verts(self):
        return (self.res + 1) ** 3

    @property
    def n_tets(self):
        return 5 * self.res ** 3


def _rand_unit(rng):
    v = rng.normal(size=3)
    return v / np.sqrt(np.dot(v, v))


def _plane(point, normal):
    return {"type": "plane", "point": list(map(float, point)), "normal": list(map(float, normal))}


def workload_ia_small(seed=1, res=20):
    """Plain implicit arrangement: 5 random planes (unit normal, offset U[-0.5,0.5]) and
    5 spheres |x-c|-r (flipped spheres), c ~ U[-0.7,0.7]^3, r ~ U[0.2,0.6]; tet5 grid over
    [-1,1]^3."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(5):
        n = _rand_unit(rng)
        d = rng.uniform(-0.5, 0.5)
        specs.append(_plane(-d * n, n))
    for _ in range(5):
        specs.append({"type": "sphere", "center": list(rng.uniform(-0.7, 0.7, 3)), "radius": float(rng.uniform(0.2, 0.6)),
                      "is_flipped": True})
    return Workload("ia-planes-spheres-res%d" % res, "ia", res, make_functions(specs), meta={"seed": seed})


def workload_mi(seed=2, res=64, n_mat=8):
    """Material interface: f_i(x) = w_i - |x - s_i| (a sphere of radius w_i), s_i ~ U[-0.8,0.8]^3,
    w_i ~ U[0,0.2]."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(n_mat):
        specs.append({"type": "sphere", "center": list(rng.uniform(-0.8, 0.8, 3)),
                      "radius": float(rng.uniform(0.0, 0.2))})
    return Workload("mi-power-diagram-res%d" % res, "mi", res, make_functions(specs), meta={"seed": seed})


def workload_ia_degenerate(seed=3, res=128):
    """Large degenerate implicit arrangement: 8 planes, 8 spheres, 8 cylinders, 8 tori.

    Planes 0-1 have random normals and pass exactly through a random grid vertex; planes 2-3
    are axis-aligned through grid coordinates (exact zeros on whole grid layers); planes 4-7 are
    exact duplicates of planes 0-3.
    """
    rng = np.random.default_rng(seed)
    xs, ys, zs = grid_coords(res)
    specs = []
    base = []
    for a in range(2):
        i, j, k = rng.integers(res // 4, 3 * res // 4, size=3)
        base.append(_plane((xs[i], ys[j], zs[k]), _rand_unit(rng)))
    i = int(rng.integers(res // 4, 3 * res // 4))
    base.append(_plane((xs[i], ys[0], zs[0]), (1.0, 0.0, 0.0)))
    j = int(rng.integers(res // 4, 3 * res // 4))
    base.append(_plane((xs[0], ys[j], zs[0]), (0.0, 1.0, 0.0)))
    specs += base + [dict(b) for b in base]
    for _ in range(8):
        specs.append({"type": "sphere", "center": list(rng.uniform(-0.7, 0.7, 3)), "radius": float(rng.uniform(0.2, 0.6))})
    for _ in range(8):
        specs.append({"type": "cylinder", "axis_point": list(rng.uniform(-0.5, 0.5, 3)),
                      "axis_vector": list(_rand_unit(rng)), "radius": float(rng.uniform(0.1, 0.4))})
    for _ in range(8):
        specs.append({"type": "torus", "center": list(rng.uniform(-0.5, 0.5, 3)), "axis_vector": list(_rand_unit(rng)),
                      "major_radius": float(rng.uniform(0.3, 0.6)), "minor_radius": float(rng.uniform(0.05, 0.2))})
    return Workload("ia-degenerate-32func-res%d" % res, "ia", res, make_functions(specs), meta={"seed": seed})


def random_function_spec(rng, kind):
    """One function of the given kind with the parameter distributions of the workloads above."""
    if kind == "plane":
        n = _rand_unit(rng)
        return _plane(-rng.uniform(-0.5, 0.5) * n, n)
    if kind == "sphere":
        return {"type": "sphere", "center": list(rng.uniform(-0.7, 0.7, 3)), "radius": float(rng.uniform(0.2, 0.6))}
    if kind == "cylinder":
        return {"type": "cylinder", "axis_point": list(rng.uniform(-0.5, 0.5, 3)), "axis_vector": list(_rand_unit(rng)),
                "radius": float(rng.uniform(0.1, 0.4))}
    return {"type": "torus", "center": list(rng.uniform(-0.5, 0.5, 3)), "axis_vector": list(_rand_unit(rng)),
            "major_radius": float(rng.uniform(0.3, 0.6)), "minor_radius": float(rng.uniform(0.05, 0.2))}


@dataclass
class BatchWorkload:
    name: str
    mode: str
    problems: list  # (res, funcs) pairs

    @property
    def n_tets(self):
        return sum(5 * r ** 3 for r, _ in self.problems)

    @property
    def n_verts(self):
        return sum((r + 1) ** 3 for r, _ in self.problems)


def workload_batch(seed=4, n=4096, mode="ia", verts_per_axis=(9, 33), funcs=(2, 24)):
    """Batched form: n independent grids over [-1,1]^3 with vertices per axis uniform in
    verts_per_axis, a function count uniform in `funcs` and the function kinds uniform over
    plane / sphere / cylinder / torus."""
    rng = np.random.default_rng(seed)
    kinds = ["plane", "sphere", "cylinder", "torus"]
    probs = []
    for _ in range(n):
        res = int(rng.integers(verts_per_axis[0], verts_per_axis[1] + 1)) - 1
        F = int(rng.integers(funcs[0], funcs[1] + 1))
        specs = [random_function_spec(rng, kinds[int(rng.integers(0, 4))]) for _ in range(F)]
        probs.append((res, make_functions(specs)))
    return BatchWorkload("batch-%d-grids" % n, mode, probs)


def random_csg_tree(rng, n_func, depth=4):
    """A random CSG tree (units {op, a, b}: 0 intersection, 1 union, 2 negation) of depth <= `depth`
    over functions 0..n_func-1, unit 1 the root."""
    units = []

    def node(d):
        if d >= depth or rng.random() < 0.3:
            return -int(rng.integers(0, n_func)) - 1
        op = int(rng.choice([0, 1, 1, 2]))
        units.append(None)
        me = len(units)
        a = node(d + 1)
        b = node(d + 1) if op != 2 else 0
        units[me - 1] = (op, a, b)
        return me

    root = node(0)
    if root < 0:  # a lone function: wrap it so that unit 1 exists
        return [(1, root, root)]
    return units


@dataclass
class Request:
    kind: str  # "ia", "mi" or "csg"
    res: int
    funcs: np.ndarray
    tree: list = None

    @property
    def n_tets(self):
        return 5 * self.res ** 3


def workload_serve(seed=5, n=1000, tets=(10_000, 2_000_000), funcs=(2, 16), mix=(0.6, 0.3, 0.1)):
    """Served form: requests of the three kinds, tet counts log-uniform in `tets` (grid resolution
    rounded from it), function counts uniform in `funcs`."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        u = rng.random()
        kind = "ia" if u < mix[0] else ("mi" if u < mix[0] + mix[1] else "csg")
        T = float(np.exp(rng.uniform(np.log(tets[0]), np.log(tets[1]))))
        res = max(1, int(round((T / 5.0) ** (1.0 / 3.0))))
        F = int(rng.integers(funcs[0], funcs[1] + 1))
        tree = None
        if kind == "mi":
            specs = [{"type": "sphere", "center": list(rng.uniform(-0.8, 0.8, 3)),
                      "radius": float(rng.uniform(0.0, 0.2))} for _ in range(F)]
        elif kind == "csg":
            specs = [random_function_spec(rng, ["sphere", "cylinder"][int(rng.integers(0, 2))]) for _ in range(F)]
            tree = random_csg_tree(rng, F)
        else:
            kinds = ["plane", "sphere", "cylinder", "torus"]
            specs = [random_function_spec(rng, kinds[int(rng.integers(0, 4))]) for _ in range(F)]
        out.append(Request(kind, res, make_functions(specs), tree))
    return out


WORKLOADS = {
    "ia-small": workload_ia_small,
    "mi": workload_mi,
    "ia-degenerate": workload_ia_degenerate,
}
