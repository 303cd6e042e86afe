"""The reference's paper examples on the GPU, whole grids through every stage against the oracle:
Fig19's inverse-CSG models (16 to 26 planes, cylinders and tori; examples/Fig19_teaser_left) and
Fig16's 18 spheres in both modes (examples/Fig16), each on its own grid, box and lookup switches
(tests/golden/examples, extracted by make_examples.py).  Combinatorics, per-tet records included, bit
for bit; coordinates within 1e-12 relative."""
import json
import os

import numpy as np
import pytest

from test_gpu_ia import assert_mesh_equal

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
EXAMPLES = os.path.join(HERE, "golden", "examples")
MANIFEST = json.load(open(os.path.join(EXAMPLES, "manifest.json")))


@pytest.fixture(scope="module")
def lib(pkg):
    pkg.build()
    return pkg.load()


@pytest.mark.parametrize("case", MANIFEST, ids=lambda e: e["file"][:-5])
def test_paper_example_every_stage(pkg, fns, oracle, lib, case):
    funcs = fns.make_functions(json.load(open(os.path.join(EXAMPLES, case["file"]))))
    res = case["resolution"]
    bmin, bmax = case["bbox"]
    grid = pkg.grid_implicit_arrangement if case["mode"] == "ia" else pkg.grid_material_interface
    mesh = grid(res, funcs, bbox_min=bmin, bbox_max=bmax, use_lookup=case["use_lookup"],
                use_secondary_lookup=case["use_secondary_lookup"])
    pts, tets = fns.generate_tet_mesh(res, bmin, bmax)
    fv = oracle.sample(funcs, pts, threads=os.cpu_count() or 1)
    assert np.array_equal(mesh["func_vals"].reshape(fv.shape), fv)
    ref = oracle.run(case["mode"], pts, tets, fv, threads=os.cpu_count() or 1)
    assert ref["stats_named"]["num_intersecting_tet"] > 0
    assert_mesh_equal(mesh, ref)
