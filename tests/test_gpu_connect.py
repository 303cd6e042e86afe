"""Mesh connectivity on the device (src/mesh_connectivity.cpp:10-242: compute_mesh_edges,
compute_patches, compute_chains) and the local-to-global maps of the extraction variants
(src/extract_mesh.cpp:268-566, 988-1443) against the oracle, bit for bit: edge numbering by first
occurrence in face order, each edge's occurrences, each face corner's edge, the patches and chains
with their faces and edges in the reference's breadth-first order, and the patch labels."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CONN = ("edges", "edge_face_offsets", "edge_faces", "face_edges", "patch_offsets", "patch_faces", "chain_offsets",
        "chain_edges")


@pytest.fixture(scope="module")
def lib(pkg):
    pkg.build()
    return pkg.load()


def assert_connectivity_equal(mesh, ref, mode):
    for k in CONN:
        a, b = mesh[k], ref[k].reshape(mesh[k].shape) if ref[k].size else ref[k]
        assert a.size == b.size and np.array_equal(a.reshape(-1), b.reshape(-1)), k
    want = ref["patch_label"].copy()
    if mode == "ia":
        want[:, 1] = -1
    assert np.array_equal(mesh["patch_label"], want)


def _grid_case(fns, name, res):
    if name == "ia-degenerate":
        wl = fns.workload_ia_degenerate(res=res)
        return "ia", wl.funcs
    if name == "mi":
        return "mi", fns.workload_mi(res=res).funcs
    mode, fn = name.split(":")
    return mode, fns.load_functions(os.path.join(GOLDEN, "functions", fn + ".json"))


@pytest.mark.parametrize("name,res", [("ia-degenerate", 24), ("ia-degenerate", 64), ("mi", 24), ("mi", 48),
                                      ("ia:3-sphere-3", 101), ("ia:2-planesphere", 101), ("mi:3-sphere-1", 101)])
def test_grid_connectivity_and_maps(pkg, fns, oracle, lib, name, res):
    mode, funcs = _grid_case(fns, name, res)
    grid = pkg.grid_implicit_arrangement if mode == "ia" else pkg.grid_material_interface
    mesh = grid(res, funcs)
    pts, tets = fns.generate_tet_mesh(res)
    fv = oracle.sample(funcs, pts, threads=os.cpu_count() or 1)
    ref = oracle.run(mode, pts, tets, fv, threads=os.cpu_count() or 1, connectivity=True)
    assert_connectivity_equal(mesh, ref, mode)
    for k in ("tet_vert_offsets", "tet_verts", "tet_face_offsets", "tet_faces"):
        assert np.array_equal(mesh[k], ref[k]), k


def test_degenerate_ties_maps_and_connectivity(pkg, fns, oracle, lib):
    """Integer materials with exact ties on explicit tets: material-interface faces on the tet
    boundary (named in both tets in the face map), non-manifold edges and chains."""
    rng = np.random.default_rng(4)
    pts, tets = fns.generate_tet_mesh(6)
    both = 0
    for _ in range(5):
        fv = rng.integers(-2, 3, size=(len(pts), 4)).astype(np.float64)
        fv[:, 3] = fv[:, 1]
        mesh = pkg.material_interface(pts, tets, fv)
        ref = oracle.run("mi", pts, tets, fv, connectivity=True)
        assert_connectivity_equal(mesh, ref, "mi")
        for k in ("tet_vert_offsets", "tet_verts", "tet_face_offsets", "tet_faces"):
            assert np.array_equal(mesh[k], ref[k]), k
        tf = mesh["tet_faces"]
        both += int((np.bincount(tf[tf >= 0]) == 2).sum())
    assert both > 0


def test_eight_sphere_mesh(pkg, fns, oracle, lib):
    m = np.load(os.path.join(GOLDEN, "mesh_8sphere.npz"))
    funcs = fns.load_functions(os.path.join(GOLDEN, "functions", "8-sphere.json"))
    fv = oracle.sample(funcs, m["pts"])
    mesh = pkg.material_interface(m["pts"], m["tets"], fv)
    ref = oracle.run("mi", m["pts"], m["tets"], fv, connectivity=True)
    assert_connectivity_equal(mesh, ref, "mi")


def test_empty_mesh(pkg, fns, lib):
    """A function with no zero crossing in the grid: no faces, no edges, no patches or chains."""
    funcs = fns.make_functions([{"type": "plane", "point": [5.0, 0.0, 0.0], "normal": [1.0, 0.0, 0.0]}])
    mesh = pkg.grid_implicit_arrangement(4, funcs)
    assert mesh["edges"].size == 0 and mesh["patch_faces"].size == 0 and mesh["chain_edges"].size == 0
    assert mesh["patch_offsets"].tolist() == [0] and mesh["chain_offsets"].tolist() == [0]
    assert mesh["tet_verts"].size == 0 and mesh["tet_vert_offsets"].tolist() == [0] * (5 * 4 ** 3 + 1)


def test_connectivity_at_the_large_config(pkg, fns, oracle, lib):
    """The large degenerate workload (10.5M tets): every field against the oracle, and the device
    time of the connectivity build."""
    wl = fns.workload_ia_degenerate(res=128)
    mesh = pkg.grid_implicit_arrangement(wl.res, wl.funcs)
    pts, tets = fns.generate_tet_mesh(wl.res)
    fv = mesh["func_vals"].reshape(len(pts), len(wl.funcs))
    ref = oracle.run("ia", pts, tets, fv, threads=os.cpu_count() or 1, connectivity=True)
    assert_connectivity_equal(mesh, ref, "ia")
