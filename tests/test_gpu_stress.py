"""The robustness sets (tests/golden/stress, from the reference's examples/Table2_Fig11): four
spheres, or spheres and a zero function, whose centres differ by 1e-7 to 1e-6, on the sets' own
99^3-cube grid.  Every stage against the oracle, bit for bit, one instance per noise level and mode."""
import json
import os

import numpy as np
import pytest

from test_gpu_ia import assert_mesh_equal

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
STRESS = os.path.join(HERE, "golden", "stress")


def _cases():
    seen, out = set(), []
    for e in json.load(open(os.path.join(STRESS, "manifest.json"))):
        if (e["mode"], e["noise"]) not in seen:
            seen.add((e["mode"], e["noise"]))
            out.append(e)
    return out


@pytest.fixture(scope="module")
def lib(pkg):
    pkg.build()
    return pkg.load()


@pytest.mark.parametrize("case", _cases(), ids=lambda e: e["file"][:-5])
def test_stress_set_every_stage(pkg, fns, oracle, lib, case):
    funcs = fns.make_functions(json.load(open(os.path.join(STRESS, case["file"]))))
    res = case["resolution"]
    bmin, bmax = case["bbox"]
    grid = pkg.grid_implicit_arrangement if case["mode"] == "ia" else pkg.grid_material_interface
    mesh = grid(res, funcs, bbox_min=bmin, bbox_max=bmax)
    pts, tets = fns.generate_tet_mesh(res, bmin, bmax)
    fv = oracle.sample(funcs, pts, threads=os.cpu_count() or 1)
    assert np.array_equal(mesh["func_vals"].reshape(fv.shape), fv)
    assert_mesh_equal(mesh, oracle.run(case["mode"], pts, tets, fv, threads=os.cpu_count() or 1))


def _all_cases():
    return json.load(open(os.path.join(STRESS, "manifest.json")))


@pytest.mark.parametrize("case", _all_cases(), ids=lambda e: e["file"][:-5])
def test_stress_set_robust_mode(pkg, fns, lib, case):
    """-R on every instance of the robustness sets, the inputs the reference's robustness test was
    made for (src/implicit_arrangement.cpp:137-243, src/material_interface.cpp:174-287): every active
    tet is cut in both row orders with exact predicates, and no tet fails in either order or differs
    in its vertex, face or cell counts."""
    funcs = fns.make_functions(json.load(open(os.path.join(STRESS, case["file"]))))
    res = case["resolution"]
    bmin, bmax = case["bbox"]
    grid = pkg.grid_implicit_arrangement if case["mode"] == "ia" else pkg.grid_material_interface
    st = grid(res, funcs, bbox_min=bmin, bbox_max=bmax, robust_test=True).stats
    assert st["num_intersecting_tet"] > 0
    assert (st["robust_failures"], st["robust_type2"], st["robust_type3"]) == (0, 0, 0)
