"""GPU parity of the material-interface path against the CPU oracle (through the C ABI)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from test_gpu_ia import assert_mesh_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(pkg):
    pkg.build()
    return pkg.load()


@pytest.mark.parametrize("res,use_lookup", [(20, True), (20, False), (64, True)])
def test_grid_material_workload(pkg, fns, oracle, lib, res, use_lookup):
    wl = fns.workload_mi(res=res)
    mesh = pkg.grid_material_interface(wl.res, wl.funcs, use_lookup=use_lookup)
    pts, tets = fns.generate_tet_mesh(wl.res)
    fv = oracle.sample(wl.funcs, pts, threads=os.cpu_count() or 1)
    assert np.array_equal(mesh["func_vals"].reshape(fv.shape), fv)
    assert_mesh_equal(mesh, oracle.run("mi", pts, tets, fv, threads=os.cpu_count() or 1))


def test_eight_spheres_custom_mesh(pkg, fns, oracle, lib):
    """The reference's 8-sphere known-answer mesh (tests/test_implicit_networks.cpp:685-731)."""
    m = np.load(os.path.join(GOLDEN, "mesh_8sphere.npz"))
    funcs = fns.load_functions(os.path.join(GOLDEN, "functions", "8-sphere.json"))
    fv = oracle.sample(funcs, m["pts"])
    mesh = pkg.material_interface(m["pts"], m["tets"], fv)
    assert_mesh_equal(mesh, oracle.run("mi", m["pts"], m["tets"], fv))


@pytest.mark.parametrize("name", ["3-sphere-1", "2-planesphere"])
def test_known_answer_grids(pkg, fns, oracle, lib, name):
    funcs = fns.load_functions(os.path.join(GOLDEN, "functions", name + ".json"))
    mesh = pkg.grid_material_interface(101, funcs)
    pts, tets = fns.generate_tet_mesh(101)
    fv = oracle.sample(funcs, pts, threads=os.cpu_count() or 1)
    assert_mesh_equal(mesh, oracle.run("mi", pts, tets, fv, threads=os.cpu_count() or 1))


def test_degenerate_ties(pkg, fns, oracle, lib):
    """Integer-valued materials on a small grid: exact ties at vertices, identical materials,
    boundary faces that become interfaces."""
    rng = np.random.default_rng(4)
    pts, tets = fns.generate_tet_mesh(6)
    for _ in range(5):
        fv = rng.integers(-2, 3, size=(len(pts), 4)).astype(np.float64)
        fv[:, 3] = fv[:, 1]  # an identical material
        mesh = pkg.material_interface(pts, tets, fv)
        assert_mesh_equal(mesh, oracle.run("mi", pts, tets, fv))


def test_batch_api_records(pkg, oracle, lib):
    rng = np.random.default_rng(5)
    rows = [rng.normal(size=(int(rng.integers(2, 6)), 4)) for _ in range(300)]
    rows += [rng.integers(-2, 3, size=(int(rng.integers(2, 5)), 4)).astype(np.float64) for _ in range(300)]
    got = pkg.compute_material_interface_batch(rows)
    for r, g in zip(rows, got):
        assert g == oracle.mi_cut(r)
