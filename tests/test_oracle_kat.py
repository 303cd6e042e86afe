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
import sys

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


with open(os.path.join(GOLDEN, "csg_kat.json")) as _f:
    CSG_KATS = json.load(_f)


def csg_oracle(oracle, fns, kat, pts, tets, threads=None):
    """The reference's CSG known-answer pipeline on the CPU: the oracle's implicit arrangement with
    its patches and chains, each patch labelled by point evaluation of the CSG tree on either side
    of one of its faces (csgcheck), then the reference's prune (src/csg.cpp:55-116)."""
    import csgcheck

    funcs = fns.load_functions(os.path.join(GOLDEN, "functions", kat["functions"] + ".json"))
    fv = oracle.sample(funcs, pts, threads=threads or os.cpu_count() or 1)
    if not kat["positive_inside"]:
        fv = -fv  # src/csg.cpp:36
    r = oracle.run("ia", pts, tets, fv, threads=threads or os.cpu_count() or 1, connectivity=True)
    fo, fvs = r["face_offsets"], r["face_verts"]
    faces = [fvs[fo[f]:fo[f + 1]].tolist() for f in range(len(fo) - 1)]
    po, pf = r["patch_offsets"], r["patch_faces"]
    patches = [pf[po[i]:po[i + 1]].tolist() for i in range(len(po) - 1)]
    co, ce = r["chain_offsets"], r["chain_edges"]
    chains = [ce[co[i]:co[i + 1]].tolist() for i in range(len(co) - 1)]
    first_tet = r["face_tets"][r["face_tet_offsets"][:-1], 0]
    label = lambda f: csgcheck.face_label(f, r["xyz"], fo, fvs, first_tet, r["face_func"], pts, tets, fv, kat["tree"])
    labels = csgcheck.patch_labels(patches, label)
    kept, sign, kept_chains, corners = csgcheck.prune(patches, labels, faces, len(r["xyz"]), chains,
                                                      r["edges"].tolist(), r["nm_degree"])
    return {"patches": kept, "sign_label": sign, "chains": kept_chains, "corners": corners, "run": r}


@pytest.mark.parametrize("kat", CSG_KATS, ids=[k["functions"] for k in CSG_KATS])
def test_csg_known_answer(kat, fns, oracle, grid101):
    """tests/test_implicit_networks.cpp:814-1034: patch, chain and corner counts and the ordered
    patch_sign_label list after the CSG prune, at 101^3 cubes with positive_inside = true."""
    pts, tets = grid101
    got = csg_oracle(oracle, fns, kat, pts, tets)
    assert len(got["patches"]) == kat["patches"]
    assert len(got["chains"]) == kat["chains"]
    assert got["corners"] == kat["corners"]
    assert got["sign_label"] == kat["sign_label"]


def test_lambda_to_tree():
    """The golden script's lambda parser builds the tree the reference's lambda describes."""
    sys.path.insert(0, GOLDEN)
    import csgcheck
    from make_golden import lambda_to_tree

    rng = np.random.default_rng(3)
    cases = {"cells_label[0] && !cells_label[0]": lambda c: c[0] and not c[0],
             "cells_label[0] || (cells_label[1] && cells_label[2])": lambda c: c[0] or (c[1] and c[2]),
             "cells_label[0] && !(cells_label[1] && cells_label[2])": lambda c: c[0] and not (c[1] and c[2]),
             "cells_label[1] || cells_label[2]": lambda c: c[1] or c[2],
             "!cells_label[2] && cells_label[0] || cells_label[1]": lambda c: (not c[2] and c[0]) or c[1],
             "cells_label[1]": lambda c: c[1]}
    for text, fn in cases.items():
        tree = lambda_to_tree(text)
        for _ in range(16):
            v = rng.choice([-1.0, 1.0], size=3)
            assert csgcheck.inside(tree, v) == fn(v > 0), text
