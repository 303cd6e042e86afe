"""The C++ host layer and its command-line programs on the GPU (app/implicit_arrangement.cpp and
app/material_interface.cpp of the reference): mesh.json, stats.json and timings.json against the
oracle, and the reference's known answers (tests/test_implicit_networks.cpp) through the programs."""
import json
import os
import shutil
import subprocess
from collections import Counter

import numpy as np
import pytest

import meshjson
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(REPO, "robust-implicit-surface-networks_gb300", "_build")
APP = {"ia": "impl_arrangement", "mi": "material_interface"}

with open(os.path.join(GOLDEN, "kat.json")) as _f:
    KATS = json.load(_f)


@pytest.fixture(scope="module")
def built(pkg):
    pkg.build()
    return BIN


def _config(tmp_path, name, res=None, mesh_file=None, **switches):
    shutil.copy(os.path.join(GOLDEN, "functions", name + ".json"), tmp_path / "fn.json")
    os.makedirs(tmp_path / "out", exist_ok=True)
    body = {"funcFile": "fn.json", "outputDir": "out"}
    if mesh_file:
        body["tetMeshFile"] = mesh_file
    else:
        body.update({"gridResolution": res, "gridBbox": [[-1.0, -1.0, -1.0], [1.0, 1.0, 1.0]]})
    body.update(switches)
    (tmp_path / "config.json").write_text(json.dumps(body))
    return tmp_path / "config.json"


def _run(mode, cfg, *flags):
    r = subprocess.run([os.path.join(BIN, APP[mode]), str(cfg), *flags], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


@pytest.mark.parametrize("mode,name,res,lookup", [("ia", "3-sphere-3", 24, True), ("ia", "2-planesphere", 20, False),
                                                  ("mi", "3-sphere-1", 22, True), ("mi", "8-sphere", 18, False)])
def test_cli_matches_oracle(built, fns, oracle, tmp_path, mode, name, res, lookup):
    cfg = _config(tmp_path, name, res, useLookup=lookup)
    _run(mode, cfg)
    funcs = fns.load_functions(os.path.join(GOLDEN, "functions", name + ".json"))
    pts, tets = fns.generate_tet_mesh(res)
    ref = oracle.run(mode, pts, tets, oracle.sample(funcs, pts), connectivity=True)
    got = meshjson.load_mesh_json(tmp_path / "out" / "mesh.json")
    meshjson.compare(got, meshjson.expected_mesh_json(ref, mode), xyz_rtol=1e-12)
    stats = json.load(open(tmp_path / "out" / "stats.json"))
    rs = ref["stats_named"]
    tag = "iso" if mode == "ia" else "MI"
    assert stats["num_pts"] == rs["num_pts"] and stats["num_tets"] == rs["num_tets"]
    assert stats["num_intersecting_tet"] == rs["num_intersecting_tet"]
    assert stats[f"num_{tag}_verts"] == rs["num_verts"] and stats[f"num_{tag}_faces"] == rs["num_faces"]
    assert stats[f"num_{tag}_edges"] == len(ref["edges"])
    assert stats["num_patches"] == len(ref["patch_offsets"]) - 1
    assert stats["num_chains"] == len(ref["chain_offsets"]) - 1
    timings = json.load(open(tmp_path / "out" / "timings.json"))
    assert "patches" in timings and "chains" in timings and all(v >= 0 for v in timings.values())


def test_cli_tet_mesh_file(built, fns, oracle, tmp_path):
    m = np.load(os.path.join(GOLDEN, "mesh_8sphere.npz"))
    (tmp_path / "tets.json").write_text(json.dumps([m["pts"].tolist(), m["tets"].tolist()]))
    cfg = _config(tmp_path, "8-sphere", mesh_file="tets.json")
    _run("mi", cfg)
    funcs = fns.load_functions(os.path.join(GOLDEN, "functions", "8-sphere.json"))
    ref = oracle.run("mi", m["pts"], m["tets"], oracle.sample(funcs, m["pts"]), connectivity=True)
    got = meshjson.load_mesh_json(tmp_path / "out" / "mesh.json")
    meshjson.compare(got, meshjson.expected_mesh_json(ref, "mi"), xyz_rtol=1e-12)


def test_cli_flags(built, tmp_path):
    cfg = _config(tmp_path, "2-sphere", 16)
    _run("ia", cfg, "-T")
    assert not (tmp_path / "out" / "mesh.json").exists()
    assert (tmp_path / "out" / "timings.json").exists() and (tmp_path / "out" / "stats.json").exists()
    out = _run("ia", cfg, "--robust-test")
    assert "success." in out
    out = _run("mi", cfg, "-R")
    assert "success." in out


def test_cli_bad_function_file(built, tmp_path):
    cfg = _config(tmp_path, "2-sphere", 8)
    (tmp_path / "fn.json").write_text(json.dumps([{"type": "cone"}]))
    r = subprocess.run([os.path.join(BIN, APP["ia"]), str(cfg)], capture_output=True, text=True, timeout=120)
    assert r.returncode != 0 and "function loading failed." in r.stdout


def _corners(mesh):
    """Vertices with more than two incident non-manifold edges, from mesh.json alone."""
    count = Counter()
    for f in mesh["faces"] or []:
        for i in range(len(f)):
            a, b = f[i], f[(i + 1) % len(f)]
            count[(min(a, b), max(a, b))] += 1
    deg = Counter()
    for (a, b), c in count.items():
        if c > 2:
            deg[a] += 1
            deg[b] += 1
    return sum(1 for d in deg.values() if d > 2)


@pytest.mark.parametrize("kat", KATS, ids=[f"{k['mode']}-{k['functions']}" for k in KATS])
def test_cli_known_answers(built, tmp_path, kat):
    if kat["mesh"] == "mesh":
        m = np.load(os.path.join(GOLDEN, "mesh_8sphere.npz"))
        (tmp_path / "tets.json").write_text(json.dumps([m["pts"].tolist(), m["tets"].tolist()]))
        cfg = _config(tmp_path, kat["functions"], mesh_file="tets.json")
    else:
        cfg = _config(tmp_path, kat["functions"], 101)
    _run(kat["mode"], cfg)
    mesh = meshjson.load_mesh_json(tmp_path / "out" / "mesh.json")
    stats = json.load(open(tmp_path / "out" / "stats.json"))
    if "patches" in kat:
        assert stats["num_patches"] == kat["patches"] == len(mesh["patches"] or [])
    if "chains" in kat:
        assert stats["num_chains"] == kat["chains"] == len(mesh["chains"] or [])
    if "corners" in kat:
        assert _corners(mesh) == kat["corners"]
    assert mesh["patches_label"] == [kat["patch_label"]]


_OPS = {0: "Intersection", 1: "Union", 2: "Negation"}


def _run_csg_cli(tmp_path, res, tree):
    """app/csg.cpp's command line on a grid of `res` cubes with the functions in tmp_path/fn.json
    and `tree` (units [op, a, b]) as its --tree file; returns mesh.json."""
    (tmp_path / "tree.json").write_text(json.dumps([{"type": _OPS[op], "elements": [a, b]} for op, a, b in tree]))
    os.makedirs(tmp_path / "out", exist_ok=True)
    (tmp_path / "config.json").write_text(json.dumps({"gridResolution": res, "gridBbox": [[-1, -1, -1], [1, 1, 1]],
                                                       "funcFile": "fn.json", "outputDir": "out"}))
    r = subprocess.run([os.path.join(BIN, "csg"), str(tmp_path / "config.json"), "--tree", str(tmp_path / "tree.json")],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    got = json.loads(open(tmp_path / "out" / "mesh.json").read())
    assert list(got) == ["chains", "corners", "edges", "faces", "patches", "patches_label", "points"]
    return got


def _csg_expected(oracle, pts, tets, fv, tree):
    """The oracle's arrangement, patches and chains, each patch labelled by point evaluation of the
    tree (independent of the library's labels), pruned as src/csg.cpp:55-116 does."""
    import csgcheck

    ref = oracle.run("ia", pts, tets, fv, threads=os.cpu_count() or 1, connectivity=True)
    full = meshjson.expected_mesh_json(ref, "ia")
    full = {k: (v if v is not None else []) for k, v in full.items()}
    fo, fvs = ref["face_offsets"], ref["face_verts"]
    first_tet = ref["face_tets"][ref["face_tet_offsets"][:-1], 0]
    label = lambda f: csgcheck.face_label(f, ref["xyz"], fo, fvs, first_tet, ref["face_func"], pts, tets, fv, tree)
    labels = csgcheck.patch_labels(full["patches"], label)
    kept, sign, chains, corners = csgcheck.prune(full["patches"], labels, full["faces"], len(ref["xyz"]),
                                                 full["chains"] or [], ref["edges"].tolist(), ref["nm_degree"])
    return full, kept, sign, chains, corners


def _corners_after_prune(mesh):
    """The reference test's corners_count from mesh.json: vertices with more than two non-manifold
    edges, once the vertices counted at most twice in the kept patches' faces lost theirs."""
    import csgcheck

    faces = mesh["faces"] or []
    nm = csgcheck.nm_degree_from_faces(faces, len(mesh["points"] or []))
    if len(nm) == 0:
        return 0
    count = np.zeros(len(nm), dtype=np.int64)
    for p in mesh["patches"] or []:
        for f in p:
            for v in faces[f]:
                count[v] += 1
    nm[count <= 2] = 0
    return int((nm > 2).sum())


def test_cli_csg(built, fns, oracle, tmp_path):
    """app/csg.cpp through the C++ host layer: the kept patches, their sign labels and the kept
    chains equal the oracle's, labelled by point evaluation of the tree on both sides of a face."""
    specs = [{"type": "sphere", "center": [0.1, 0.0, 0.05], "radius": 0.55},
             {"type": "cylinder", "axis_point": [0.0, 0.1, 0.0], "axis_vector": [0.2, 1.0, 0.1], "radius": 0.3},
             {"type": "sphere", "center": [-0.3, 0.2, -0.1], "radius": 0.4}]
    (tmp_path / "fn.json").write_text(json.dumps(specs))
    tree = [(1, 2, -3), (0, -1, 3), (2, -2, 0)]  # (f0 - f1) | f2
    res = 20
    got = _run_csg_cli(tmp_path, res, tree)
    funcs = fns.make_functions(specs)
    pts, tets = fns.generate_tet_mesh(res)
    full, kept, sign, chains, corners = _csg_expected(oracle, pts, tets, oracle.sample(funcs, pts), tree)
    assert len(kept) > 0
    assert got["patches"] == kept
    assert got["patches_label"] == [sign]
    assert (got["chains"] or []) == chains
    assert _corners_after_prune(got) == corners
    assert got["faces"] == full["faces"] and got["edges"] == full["edges"]


with open(os.path.join(GOLDEN, "csg_kat.json")) as _f:
    CSG_KATS = json.load(_f)


@pytest.mark.parametrize("kat", CSG_KATS, ids=[k["functions"] for k in CSG_KATS])
def test_cli_csg_known_answers(built, fns, oracle, tmp_path, kat):
    """The reference's CSG known answers (tests/test_implicit_networks.cpp:814-1034) through the csg
    program (ria_host::csg, positive_inside = true) at 101^3 cubes: patch, chain and corner counts
    and the ordered patch_sign_label list; the kept patches and chains also equal the oracle's."""
    shutil.copy(os.path.join(GOLDEN, "functions", kat["functions"] + ".json"), tmp_path / "fn.json")
    got = _run_csg_cli(tmp_path, 101, kat["tree"])
    patches, chains = got["patches"] or [], got["chains"] or []
    assert len(patches) == kat["patches"]
    assert len(chains) == kat["chains"]
    assert _corners_after_prune(got) == kat["corners"]
    assert got["patches_label"] == [kat["sign_label"]]
    funcs = fns.load_functions(os.path.join(GOLDEN, "functions", kat["functions"] + ".json"))
    pts, tets = fns.generate_tet_mesh(101)
    fv = oracle.sample(funcs, pts, threads=os.cpu_count() or 1)
    _, kept, sign, kchains, corners = _csg_expected(oracle, pts, tets, fv, kat["tree"])
    assert patches == kept and chains == kchains and corners == kat["corners"]
