"""GPU parity of the implicit-arrangement path against the CPU oracle (through the C ABI).

Combinatorics (active-function CRS, per-tet records, vertex records, face lists, tet-face lists,
function labels) must be bit-exact; vertex coordinates within 1e-12 relative (they are computed with
the same operation order and in practice match exactly).
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

XYZ_RTOL = 1e-12


def assert_mesh_equal(mesh, ref, records=True, maps=True):
    """Every field of a device mesh against the oracle's; `maps`: also the local-to-global maps of the
    extraction variants (src/extract_mesh.cpp:268-566, 988-1443)."""
    for k in ("verts", "face_offsets", "face_verts", "face_tet_offsets", "face_tets", "face_func"):
        a, b = mesh[k], ref[k]
        assert a.shape == b.shape and np.array_equal(a, b), k
    if maps:
        assert not (ref["tet_verts"] == np.iinfo(np.int64).min).any(), "oracle: vertex on no face is not a corner"
        for k in ("tet_vert_offsets", "tet_verts", "tet_face_offsets", "tet_faces"):
            a, b = mesh[k], ref[k]
            assert a.shape == b.shape and np.array_equal(a, b), k
    x, y = mesh["xyz"], ref["xyz"]
    assert x.shape == y.shape
    assert np.all(np.abs(x - y) <= XYZ_RTOL * np.maximum(1.0, np.abs(y)))
    assert np.array_equal(mesh["start_index"], ref["start_index"])
    assert np.array_equal(mesh["func_in_tet"], ref["func_in_tet"])
    if records:
        assert np.array_equal(mesh["rec_offsets"], ref["rec_offsets"])
        assert np.array_equal(mesh["rec_bytes"], ref["rec_bytes"])
    st = mesh.stats
    assert st["robust_failures"] == st["robust_type2"] == st["robust_type3"] == 0
    rs = ref["stats_named"]
    for k in ("num_pts", "num_tets", "num_degenerate_vertex", "num_intersecting_tet", "num_a_func", "num_b_func",
              "num_more_func", "num_verts", "num_faces"):
        assert st[k] == rs[k], k


@pytest.fixture(scope="module")
def lib(pkg):
    pkg.build()
    return pkg.load()


def test_sampling_bit_exact(pkg, fns, oracle, lib):
    rng = np.random.default_rng(1)
    specs = [
        {"type": "plane", "point": [0.1, -0.2, 0.3], "normal": [0.3, 0.5, -0.8]},
        {"type": "sphere", "center": [0.1, 0.2, -0.1], "radius": 0.4},
        {"type": "sphere", "center": [0.1, 0.2, -0.1], "radius": 0.4, "squared": True, "is_flipped": True},
        {"type": "cylinder", "axis_point": [0.0, 0.1, 0.2], "axis_vector": [1.0, 2.0, 3.0], "radius": 0.3},
        {"type": "torus", "center": [0.0, 0.1, 0.2], "axis_vector": [0.2, -1.0, 0.4], "major_radius": 0.5,
         "minor_radius": 0.1},
        {"type": "zero"},
    ]
    funcs = fns.make_functions(specs)
    pts = rng.uniform(-1, 1, size=(50000, 3))
    assert np.array_equal(pkg.sample_functions(funcs, pts), oracle.sample(funcs, pts))


def test_sampling_square_roots_wide_range(pkg, fns, oracle, lib):
    """The device's integer square root over the whole exponent range: points from 1e-170 to 1e170
    (subnormal and infinite sums of squares included) through the spheres, cylinder and torus,
    bit for bit against the oracle's C library sqrt."""
    rng = np.random.default_rng(17)
    specs = [
        {"type": "sphere", "center": [0.0, 0.0, 0.0], "radius": 1.0},
        {"type": "sphere", "center": [1e-3, -2e-3, 5e-4], "radius": 0.5},
        {"type": "cylinder", "axis_point": [0.0, 0.0, 0.0], "axis_vector": [0.3, -0.4, 0.5], "radius": 0.3},
        {"type": "torus", "center": [0.0, 0.0, 0.0], "axis_vector": [0.0, 0.0, 1.0], "major_radius": 0.5,
         "minor_radius": 0.1},
    ]
    funcs = fns.make_functions(specs)
    pts = rng.uniform(-1, 1, size=(400000, 3)) * 10.0 ** rng.uniform(-170, 170, size=(400000, 1))
    got, want = pkg.sample_functions(funcs, pts), oracle.sample(funcs, pts)
    assert np.array_equal(got, want, equal_nan=True)


@pytest.mark.parametrize("use_lookup", [True, False])
def test_grid_small_workload(pkg, fns, oracle, lib, use_lookup):
    wl = fns.workload_ia_small()
    mesh = pkg.grid_implicit_arrangement(wl.res, wl.funcs, use_lookup=use_lookup)
    pts, tets = fns.generate_tet_mesh(wl.res)
    fv = oracle.sample(wl.funcs, pts)
    assert np.array_equal(mesh["func_vals"].reshape(fv.shape), fv)
    assert_mesh_equal(mesh, oracle.run("ia", pts, tets, fv))


def test_host_buffers_custom_mesh(pkg, fns, oracle, lib):
    m = np.load(os.path.join(GOLDEN, "mesh_8sphere.npz"))
    funcs = fns.load_functions(os.path.join(GOLDEN, "functions", "8-sphere.json"))
    fv = oracle.sample(funcs, m["pts"])
    mesh = pkg.implicit_arrangement(m["pts"], m["tets"], fv)
    assert_mesh_equal(mesh, oracle.run("ia", m["pts"], m["tets"], fv))


@pytest.mark.parametrize("name", ["2-planesphere", "3-sphere-3", "1-plane"])
def test_known_answer_fixtures(pkg, fns, oracle, lib, name):
    """The reference's known-answer grids (101^3 cubes); the oracle's output there is pinned to the
    reference's patch/chain counts by test_oracle_kat.py."""
    funcs = fns.load_functions(os.path.join(GOLDEN, "functions", name + ".json"))
    mesh = pkg.grid_implicit_arrangement(101, funcs)
    pts, tets = fns.generate_tet_mesh(101)
    fv = oracle.sample(funcs, pts, threads=os.cpu_count() or 1)
    assert_mesh_equal(mesh, oracle.run("ia", pts, tets, fv, threads=os.cpu_count() or 1))


@pytest.mark.parametrize("res", [24, 128])
def test_degenerate_workload(pkg, fns, oracle, lib, res):
    """32 functions with duplicated planes and planes through grid vertices (exact zeros)."""
    wl = fns.workload_ia_degenerate(res=res)
    mesh = pkg.grid_implicit_arrangement(wl.res, wl.funcs)
    pts, tets = fns.generate_tet_mesh(wl.res)
    fv = oracle.sample(wl.funcs, pts, threads=os.cpu_count() or 1)
    assert np.array_equal(mesh["func_vals"].reshape(fv.shape), fv)
    assert_mesh_equal(mesh, oracle.run("ia", pts, tets, fv, threads=os.cpu_count() or 1))


def test_vertex_coordinates_bit_identical(pkg, fns, oracle, lib):
    """The vertex coordinates divide on the integer pipe (div_rn.cuh) with the reference's formula
    order: the same bits as the oracle's C arithmetic, for edge, face and interior vertices (implicit
    arrangement) and for the material interface."""
    seen = set()
    for mode, wl in (("ia", fns.workload_ia_degenerate(res=24)), ("mi", fns.workload_mi(res=24)),
                     ("ia", fns.workload_ia_small(res=16))):
        run = pkg.grid_implicit_arrangement if mode == "ia" else pkg.grid_material_interface
        mesh = run(wl.res, wl.funcs)
        pts, tets = fns.generate_tet_mesh(wl.res)
        fv = oracle.sample(wl.funcs, pts)
        ref = oracle.run(mode, pts, tets, fv)
        assert np.array_equal(mesh["verts"], ref["verts"])
        assert np.array_equal(mesh["xyz"].view(np.uint64), ref["xyz"].view(np.uint64)), mode
        seen.update(np.unique(ref["verts"].reshape(-1, 11)[:, 2]).tolist())
        mesh.close()
    assert {2, 3} <= seen


@pytest.mark.parametrize("seed,nplanes,res", [(7, 20, 6), (11, 18, 6)])
def test_dense_planes_overflow_tight_tables(pkg, fns, oracle, lib, seed, nplanes, res):
    """Many planes on a small grid: vertices where two planes cross a tet face (keyed by the face
    table) outnumber the extraction's tight table (a slot per 16 vertex occurrences, at least 1,024),
    so its inserts overflow and the call runs the extraction again with worst-case tables.  The mesh
    must still equal the oracle's."""
    rng = np.random.default_rng(seed)
    funcs = fns.make_functions([fns.random_function_spec(rng, "plane") for _ in range(nplanes)])
    mesh = pkg.grid_implicit_arrangement(res, funcs)
    pts, tets = fns.generate_tet_mesh(res)
    fv = oracle.sample(funcs, pts)
    ref = oracle.run("ia", pts, tets, fv)
    occurrences = int(ref["tet_vert_offsets"][-1])  # iso vertex occurrences, as the extraction counts them
    cap = 1024
    while cap < occurrences // 16 + 1:
        cap *= 2
    assert (ref["verts"].reshape(-1, 11)[:, 2] == 3).sum() > cap
    assert_mesh_equal(mesh, ref)


def test_batch_api_records(pkg, oracle, lib):
    rng = np.random.default_rng(3)
    rows = []
    for _ in range(300):
        k = int(rng.integers(1, 6))
        rows.append(rng.normal(size=(k, 4)))
    for _ in range(300):
        k = int(rng.integers(1, 5))
        rows.append(rng.integers(-2, 3, size=(k, 4)).astype(np.float64))
    got = pkg.compute_arrangement_batch(rows)
    for r, g in zip(rows, got):
        assert g == oracle.ia_cut(r)


def test_robust_mode(pkg, fns, lib):
    """-R on a grid (src/implicit_arrangement.cpp:137-243): no tet of any failure type, and the
    per-count statistics of the tets the robust pass cut equal the normal pass's."""
    wl = fns.workload_ia_degenerate(res=24)
    mesh = pkg.grid_implicit_arrangement(wl.res, wl.funcs, robust_test=True)
    st = mesh.stats
    assert st["robust_failures"] == 0 and st["robust_type2"] == 0 and st["robust_type3"] == 0
    ref = pkg.grid_implicit_arrangement(wl.res, wl.funcs).stats
    for k in ("num_intersecting_tet", "num_a_func", "num_b_func", "num_more_func", "num_degenerate_vertex"):
        assert st[k] == ref[k], k


def test_repeatable(pkg, fns, lib):
    wl = fns.workload_ia_degenerate(res=32)
    a = pkg.grid_implicit_arrangement(wl.res, wl.funcs)
    b = pkg.grid_implicit_arrangement(wl.res, wl.funcs)
    for k in ("verts", "face_verts", "face_tets", "xyz", "rec_bytes"):
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("mode", ["ia", "mi"])
def test_secondary_lookup_cache(pkg, fns, oracle, lib, mode):
    """Two-plane (IA) / three-material (MI) tets come from the device cache of records keyed by
    their combinatorial type once seen.  The first call fills the cache, the second reads it; both
    equal the general cut (useSecondaryLookup off) and the oracle."""
    if mode == "ia":
        wl = fns.workload_ia_degenerate(res=40)
        grid = pkg.grid_implicit_arrangement
    else:
        wl = fns.workload_mi(res=40)
        grid = pkg.grid_material_interface
    pts, tets = fns.generate_tet_mesh(wl.res)
    fv = oracle.sample(wl.funcs, pts)
    ref = oracle.run(mode, pts, tets, fv)
    off = grid(wl.res, wl.funcs, use_secondary_lookup=False)
    for _ in range(2):
        on = grid(wl.res, wl.funcs, use_secondary_lookup=True)
        assert_mesh_equal(on, ref)
        for k in ("rec_bytes", "verts", "face_verts", "xyz"):
            assert np.array_equal(on[k], off[k]), k


@pytest.mark.parametrize("mode", ["ia", "mi"])
def test_heavy_single_tets_through_extraction(pkg, fns, oracle, lib, mode):
    """Single tets whose arrangements exceed 128 vertices and 64 cells (the exact variant's range
    reaches 255 / 254), through sampling-free host entry points, filter, cut and extraction."""
    rng = np.random.default_rng(80)
    pts = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
    tets = np.array([[0, 1, 2, 3]])
    big = 0
    for it in range(16):
        if mode == "ia":
            k = int(rng.integers(9, 15))
            fv = rng.normal(size=(4, k))
        else:
            # every material owns a cell: tangent planes of |x|^2 at sites inside the tet (Voronoi)
            k = int(rng.integers(30, 45))
            sites = rng.dirichlet(np.ones(4), size=k) @ pts
            fv = np.stack([2 * pts @ c - c @ c for c in sites], axis=1)
        call = pkg.implicit_arrangement if mode == "ia" else pkg.material_interface
        try:
            mesh = call(pts, tets, fv)
        except pkg.RiaError as e:
            assert e.status == pkg._lib.RIA_ECAPACITY
            continue
        ref = oracle.run(mode, pts, tets, fv)
        assert_mesh_equal(mesh, ref)
        big += int(len(mesh["verts"]) > 128)
    assert big > 0
