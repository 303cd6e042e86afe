"""Pin the oracle against the reference's own known-answer tests (CPU only).

tests/golden/kat.json is extracted from tests/test_implicit_networks.cpp by
tests/golden/make_golden.py.  The reference checks, after its downstream stages, the patch count,
chain count, corner count and the ordered patch_function_label list.  The oracle restates the
stages that produce those numbers (src/mesh_connectivity.cpp:10-242) on top of stages (a)-(d), so
the comparison pins the filter, the per-tet cut, the first-occurrence numbering of
extract_mesh and the sampler's sign conventions.  Arrangement cells and shells need the
out-of-scope nesting stages and are not compared.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

with open(os.path.join(GOLDEN, "kat.json")) as _f:
    KATS = json.load(_f)


@pytest.fixture(scope="module")
def grid101(fns):
    return fns.generate_tet_mesh(101)


@pytest.mark.parametrize("kat", KATS, ids=[f"{k['mode']}-{k['functions']}" for k in KATS])
def test_known_answer(kat, fns, oracle, grid101):
    if kat["mesh"] == "mesh":
        m = np.load(os.path.join(GOLDEN, "mesh_8sphere.npz"))
        pts, tets = m["pts"], m["tets"]
    else:
        pts, tets = grid101
    funcs = fns.load_functions(os.path.join(GOLDEN, "functions", kat["functions"] + ".json"))
    fv = oracle.sample(funcs, pts, threads=os.cpu_count() or 1)
    if kat["mode"] == "mi" and fv.shape[1] < 2:
        # a single material has no interface: the reference expects no patches and no chains
        assert kat["patches"] == 0 and kat.get("chains", 0) == 0
        return
    r = oracle.run(kat["mode"], pts, tets, fv, threads=os.cpu_count() or 1, connectivity=True)
    n_patch = len(r["patch_offsets"]) - 1
    if "patches" in kat:
        assert n_patch == kat["patches"]
    if "chains" in kat:
        assert len(r["chain_offsets"]) - 1 == kat["chains"]
    if "corners" in kat:
        assert int((r["nm_degree"] > 2).sum()) == kat["corners"]
    if kat["mode"] == "ia":
        assert r["patch_label"][:, 0].tolist() == kat["patch_label"]
    else:
        assert r["patch_label"].tolist() == kat["patch_label"]
