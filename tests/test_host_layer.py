"""The CPU half of the C++ host layer (host/mesh_io.cpp) against the Python host code and the oracle:
tet grid, readers, connectivity and the mesh.json writer (src/io.cpp, src/mesh_connectivity.cpp)."""
import json
import os
import struct
import subprocess

import numpy as np
import pytest

import meshjson

HERE = os.path.dirname(os.path.abspath(__file__))
# RIA_MESHIO_CHECK: another build of the same sources (the sanitizer builds of `make sanitize`)
CHECK = os.environ.get("RIA_MESHIO_CHECK") or os.path.join(HERE, "hostcheck", "_build", "meshio_check")


@pytest.fixture(scope="module")
def check():
    subprocess.run(["make", "-C", os.path.join(HERE, "hostcheck"), "-s"], check=True)
    return CHECK


def _run(*args):
    return subprocess.run([CHECK, *map(str, args)], capture_output=True, text=True, check=True).stdout


@pytest.mark.parametrize("res,lo,hi", [(1, (-1, -1, -1), (1, 1, 1)), (7, (-1, -1, -1), (1, 1, 1)),
                                       (6, (-0.3, 0.1, -2.5), (1.7, 0.45, 3.0))])
def test_generate_tet_mesh_matches(check, fns, tmp_path, res, lo, hi):
    out = tmp_path / "g.bin"
    _run("grid", res, *lo, *hi, out)
    pts, tets = meshjson.read_grid(out)
    p2, t2 = fns.generate_tet_mesh(res, lo, hi)
    assert np.array_equal(pts, p2) and np.array_equal(tets, t2)


def test_tet_mesh_reader(check, tmp_path):
    rng = np.random.default_rng(3)
    pts = rng.normal(size=(9, 3))
    tets = rng.integers(0, 9, size=(5, 4))
    f = tmp_path / "m.json"
    f.write_text(json.dumps([pts.tolist(), tets.tolist()]))
    out = tmp_path / "m.bin"
    _run("tetmesh", f, out)
    p2, t2 = meshjson.read_grid(out)
    assert np.array_equal(p2, pts) and np.array_equal(t2, tets)


@pytest.mark.parametrize("layout", ["compact", "indented", "extra_values", "float_indices"])
def test_tet_mesh_reader_layouts(check, fns, tmp_path, layout):
    """The streaming reader (compact or indented text) and the general parser it falls back to
    (rows with extra values, indices written as floats) give the same mesh."""
    pts, tets = fns.generate_tet_mesh(6, (-0.3, 0.1, -2.5), (1.7, 0.45, 3.0))
    P, T = pts.tolist(), tets.tolist()
    if layout == "extra_values":
        P = [p + [9.0] for p in P]
    if layout == "float_indices":
        T = [[float(v) for v in t] for t in T]
    f = tmp_path / "m.json"
    f.write_text(json.dumps([P, T], indent=2 if layout == "indented" else None))
    out = tmp_path / "m.bin"
    _run("tetmesh", f, out)
    p2, t2 = meshjson.read_grid(out)
    assert np.array_equal(p2, pts) and np.array_equal(t2, tets)


def test_tet_mesh_reader_fuzzed_formatting(check, tmp_path):
    """Random whitespace between tokens and varied number spellings (exponents, signs, integers for
    coordinates): the reader agrees with Python's JSON parser on the same text."""
    rng = np.random.default_rng(20)
    ws = [" ", "\n", "\t", "\r\n", "  ", ""]

    def sp():
        return "".join(rng.choice(ws) for _ in range(int(rng.integers(0, 3))))

    def num(x, integer=False):
        if integer:
            return str(int(x))
        form = int(rng.integers(0, 4))
        if form == 0:
            return repr(float(x))
        if form == 1:
            return "%.17e" % x
        if form == 2:
            return ("%.17E" % x).replace("E+", "E")
        return str(int(round(x)))

    for trial in range(30):
        n_p, n_t = int(rng.integers(0, 40)), int(rng.integers(0, 60))
        pts = rng.normal(size=(n_p, 3)) * 10.0 ** rng.uniform(-8, 8, size=(n_p, 1))
        tets = rng.integers(0, max(n_p, 1), size=(n_t, 4))
        rows_p = [sp() + "[" + ",".join(sp() + num(v) + sp() for v in p) + "]" + sp() for p in pts]
        rows_t = [sp() + "[" + ",".join(sp() + num(v, True) + sp() for v in t) + "]" + sp() for t in tets]
        text = sp() + "[" + sp() + "[" + ",".join(rows_p) + "]" + sp() + "," + sp() + "[" + ",".join(rows_t) + "]" \
            + sp() + "]" + sp()
        f = tmp_path / ("m%d.json" % trial)
        f.write_text(text)
        out = tmp_path / ("m%d.bin" % trial)
        _run("tetmesh", f, out)
        p2, t2 = meshjson.read_grid(out)
        P, T = json.loads(text)
        assert np.array_equal(p2, np.array(P, dtype=np.float64).reshape(-1, 3)), trial
        assert np.array_equal(t2, np.array(T, dtype=np.int64).reshape(-1, 4)), trial


def test_tet_mesh_reader_rejects_truncated_file(check, tmp_path):
    f = tmp_path / "m.json"
    f.write_text("[[[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]], [[0, 1, 0")
    r = subprocess.run([CHECK, "tetmesh", str(f), str(tmp_path / "m.bin")], capture_output=True, text=True)
    assert r.returncode == 3 and "JSON parse error" in r.stderr


def test_function_reader_matches(check, fns, tmp_path):
    files = sorted(os.listdir(os.path.join(HERE, "golden", "functions")))
    specs = [json.load(open(os.path.join(HERE, "golden", "functions", n))) for n in files]
    specs.append([
        {"type": "plane", "point": [0.1, 0.2, 0.3], "normal": [1, -2, 0.5], "is_flipped": True},
        {"type": "sphere", "center": [0, 0.5, 0], "radius": 0.3, "squared": True},
        {"type": "cylinder", "axis_point": [0.1, 0, 0], "axis_vector": [0.3, 0.4, 1.7], "radius": 0.25},
        {"type": "torus", "center": [0, 0, 0.1], "axis_vector": [1, 1, 0.2], "major_radius": 0.6,
         "minor_radius": 0.1, "is_flipped": True},
        {"type": "zero"},
    ])
    for i, s in enumerate(specs):
        f = tmp_path / ("f%d.json" % i)
        f.write_text(json.dumps(s))
        out = tmp_path / ("f%d.bin" % i)
        _run("funcs", f, out)
        got = np.frombuffer(out.read_bytes(), dtype=fns.FUNC_DTYPE)
        assert got.tobytes() == fns.make_functions(s).tobytes(), i


def test_function_reader_rejects_unknown_type(check, tmp_path):
    f = tmp_path / "f.json"
    f.write_text(json.dumps([{"type": "cone", "apex": [0, 0, 0]}]))
    r = subprocess.run([CHECK, "funcs", str(f), str(tmp_path / "o.bin")], capture_output=True, text=True)
    assert r.returncode == 1 and "unsupported" in r.stdout


@pytest.mark.parametrize("body", [
    {"gridResolution": 33, "gridBbox": [[-1, -2, -3], [1, 2, 3.5]], "funcFile": "fn.json", "outputDir": "out",
     "useLookup": False, "useSecondaryLookup": True, "useTopoRayShooting": False},
    {"tetMeshFile": "sub/mesh.json", "funcFile": "/abs/fn.json"},
])
def test_config_reader_matches(check, fns, tmp_path, body):
    f = tmp_path / "config.json"
    f.write_text(json.dumps(body))
    lines = dict(l.split(" ", 1) for l in _run("config", f).strip().split("\n"))
    c = fns.parse_config_file(str(f))
    assert os.path.normpath(lines["func_file"]) == os.path.normpath(c.func_file)
    assert os.path.normpath(lines["output_dir"]) == os.path.normpath(c.output_dir)
    assert (os.path.normpath(lines["tet_mesh_file"]) if lines["tet_mesh_file"] else "") == \
        (os.path.normpath(c.tet_mesh_file) if c.tet_mesh_file else "")
    assert int(lines["resolution"]) == c.tet_mesh_resolution
    for k in ("use_lookup", "use_secondary_lookup", "use_topo_ray_shooting"):
        assert bool(int(lines[k])) == getattr(c, k), k
    if "gridBbox" in body:
        bb = [float(x) for x in lines["bbox"].split()]
        assert bb == list(c.tet_mesh_bbox_min) + list(c.tet_mesh_bbox_max)


def test_config_missing_file(check, tmp_path):
    r = subprocess.run([CHECK, "config", str(tmp_path / "nope.json")], capture_output=True, text=True)
    assert r.returncode == 3 and "does not exist" in r.stderr


@pytest.mark.parametrize("x", [0.0, -0.0, 1.0, 100.0, -2.5, 0.1, 1e-4, 1.5e-4, 1e-5, 0.000123, 123456789012345.0,
                               1234567890123456.0, 1e15, 1e16, 1e300, -1e-300, 5e-324, 2.0 ** 0.5, 1.0 / 3.0,
                               123.456, 0.3 - 0.1, 1e22, 9007199254740993.0])
def test_double_format_restatement(x):
    # the Python restatement of the printed form round-trips and agrees with JSON number syntax
    s = meshjson.nl_double(x)
    assert float(s) == x and (("." in s) or ("e" in s))
    assert json.loads(s) == x


def test_double_format_writer(check, tmp_path):
    """The C++ writer prints the same text for awkward doubles (exponent boundaries, subnormals)."""
    xs = [0.0, -0.0, 1.0, 100.0, -2.5, 0.1, 1e-4, 1.5e-4, 1e-5, 0.000123, 123456789012345.0, 1234567890123456.0,
          1e15, 1e16, 1e300, -1e-300, 5e-324, 2.0 ** 0.5, 1.0 / 3.0, 123.456, 0.3 - 0.1, 1e22, 9007199254740993.0]
    xs += [0.0] * (-len(xs) % 3)
    ref = {"xyz": np.array(xs), "face_offsets": np.zeros(1, np.int64), "face_verts": np.zeros(0, np.int64),
           "face_func": np.zeros(0, np.int64)}
    inp = tmp_path / "in.bin"
    meshjson.write_mesh_input(inp, ref)
    out = tmp_path / "mesh.json"
    _run("mesh", "ia", inp, out)
    text = out.read_text()
    pts = meshjson.dump(np.array(xs).reshape(-1, 3).tolist())
    assert '"points":' + pts + "," in text


def test_double_format_writer_random(check, tmp_path):
    """Random finite doubles over the whole exponent range, and values around the notation
    boundaries (1e-5, 1e-4, 1e15, 1e16) and integers: the writer prints the restatement's text."""
    rng = np.random.default_rng(21)
    bits = rng.integers(0, 2**64 - 1, size=210000, dtype=np.uint64).view(np.float64)  # > 65,536 rows: parallel chunks
    xs = [bits[np.isfinite(bits)]]
    for b in (1e-5, 1e-4, 1e15, 1e16):
        xs.append(b * rng.uniform(0.5, 2.0, size=3000) * rng.choice([-1.0, 1.0], size=3000))
    xs.append(rng.integers(-10**17, 10**17, size=3000).astype(np.float64))
    xs.append(np.round(rng.uniform(-1e6, 1e6, size=3000), int(rng.integers(0, 8))))
    x = np.concatenate(xs)
    x = np.concatenate([x, np.zeros(-len(x) % 3)])
    ref = {"xyz": x, "face_offsets": np.zeros(1, np.int64), "face_verts": np.zeros(0, np.int64),
           "face_func": np.zeros(0, np.int64)}
    inp = tmp_path / "in.bin"
    meshjson.write_mesh_input(inp, ref)
    out = tmp_path / "mesh.json"
    _run("mesh", "ia", inp, out)
    assert '"points":' + meshjson.dump(x.reshape(-1, 3).tolist()) + "," in out.read_text()


def _oracle_mesh(fns, oracle, mode, name=None, res=16, wl=None):
    if wl is None:
        spec = json.load(open(os.path.join(HERE, "golden", "functions", name + ".json")))
        funcs = fns.make_functions(spec)
    else:
        funcs = wl.funcs
        res = wl.res
    pts, tets = fns.generate_tet_mesh(res)
    fv = oracle.sample(funcs, pts)
    return oracle.run(mode, pts, tets, fv, connectivity=True)


@pytest.mark.parametrize("mode,name,res", [("ia", "3-sphere-1", 16), ("ia", "2-planesphere", 13), ("mi", "8-sphere", 12),
                                           ("mi", "3-sphere-2", 15), ("ia", "1-plane", 1)])
def test_mesh_json_writer_matches(check, fns, oracle, tmp_path, mode, name, res):
    ref = _oracle_mesh(fns, oracle, mode, name, res)
    inp = tmp_path / "in.bin"
    meshjson.write_mesh_input(inp, ref)
    out = tmp_path / "mesh.json"
    _run("mesh", mode, inp, out)
    got = meshjson.load_mesh_json(out)
    exp = meshjson.expected_mesh_json(ref, mode)
    meshjson.compare(got, exp)
    assert out.read_text() == meshjson.dump(exp) + "\n"


def test_mesh_json_writer_degenerate(check, fns, oracle, tmp_path):
    # non-manifold edges and chains: coincident planes and tori
    ref = _oracle_mesh(fns, oracle, "ia", wl=fns.workload_ia_degenerate(res=10))
    assert len(ref["chain_offsets"]) > 1
    inp = tmp_path / "in.bin"
    meshjson.write_mesh_input(inp, ref)
    out = tmp_path / "mesh.json"
    _run("mesh", "ia", inp, out)
    exp = meshjson.expected_mesh_json(ref, "ia")
    meshjson.compare(meshjson.load_mesh_json(out), exp)
    assert out.read_text() == meshjson.dump(exp) + "\n"


def test_mesh_json_writer_large_parallel(check, fns, oracle, tmp_path):
    """A mesh large enough that points, faces and edges are formatted in parallel chunks (over 65,536
    of each): the same bytes as the serial restatement, and the same edges, patches and chains as
    the oracle's connectivity."""
    wl = fns.workload_ia_degenerate(res=48)
    pts, tets = fns.generate_tet_mesh(wl.res)
    fv = oracle.sample(wl.funcs, pts, threads=4)
    ref = oracle.run("ia", pts, tets, fv, threads=4, connectivity=True)
    assert len(ref["xyz"]) > 65536 and len(ref["face_offsets"]) - 1 > 65536
    inp = tmp_path / "in.bin"
    meshjson.write_mesh_input(inp, ref)
    out = tmp_path / "mesh.json"
    _run("mesh", "ia", inp, out)
    exp = meshjson.expected_mesh_json(ref, "ia")
    assert len(exp["edges"]) > 65536
    assert out.read_text() == meshjson.dump(exp) + "\n"


@pytest.mark.parametrize("res", [12, 48])
def test_csg_writer(check, fns, oracle, tmp_path, res):
    """save_result_CSG (src/io.cpp:314-372): the IA document's shared lists without shells and cells,
    patch labels as booleans; at res 48 its large arrays take the parallel path."""
    wl = fns.workload_ia_degenerate(res=res)
    pts, tets = fns.generate_tet_mesh(wl.res)
    fv = oracle.sample(wl.funcs, pts, threads=4)
    ref = oracle.run("ia", pts, tets, fv, threads=4, connectivity=True)
    inp = tmp_path / "in.bin"
    meshjson.write_mesh_input(inp, ref)
    out = tmp_path / "mesh.json"
    _run("mesh", "csg", inp, out)
    ia = meshjson.expected_mesh_json(ref, "ia")
    n_patches = len(ia["patches"] or [])
    exp = {k: ia[k] for k in ("chains", "corners", "edges", "faces", "patches")}
    exp["patches_label"] = [[i % 3 == 0 for i in range(n_patches)]]
    exp["points"] = ia["points"]
    assert out.read_text() == meshjson.dump(exp) + "\n"


def test_mesh_json_writer_empty(check, tmp_path):
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(struct.pack("<q", 0) + struct.pack("<qq", 1, 0) + struct.pack("<q", 0) + struct.pack("<q", 0))
    out = tmp_path / "mesh.json"
    _run("mesh", "ia", inp, out)
    assert out.read_text() == ('{"cells":null,"cells_label":null,"chains":null,"corners":null,"edges":null,'
                               '"faces":null,"patches":null,"patches_label":[[]],"points":null,"shells":null}\n')
    _run("mesh", "mi", inp, out)
    assert '"patches_label":[[]]' in out.read_text() and '"cells_label":[[]]' in out.read_text()


def test_writer_reports_unwritable_path(check, tmp_path):
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(struct.pack("<q", 0) + struct.pack("<qq", 1, 0) + struct.pack("<q", 0) + struct.pack("<q", 0))
    r = subprocess.run([CHECK, "mesh", "csg", str(inp), str(tmp_path / "missing" / "mesh.json")], capture_output=True)
    assert r.returncode == 4
