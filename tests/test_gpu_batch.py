"""Batched grids (ria_grid_batch): every problem's fields equal those of its own grid call, bit for
bit, for mixed resolutions, function counts, kinds and boxes, and for degenerate inputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("xyz", "verts", "face_offsets", "face_verts", "face_tet_offsets", "face_tets", "face_func", "func_vals",
          "start_index", "func_in_tet", "rec_offsets", "rec_bytes")
STATS = ("num_pts", "num_tets", "num_degenerate_vertex", "num_intersecting_tet", "num_a_func", "num_b_func",
         "num_more_func", "num_verts", "num_faces")


@pytest.fixture(scope="module")
def lib(pkg):
    pkg.build()
    return pkg.load()


def _problems(fns, seed, n, mode):
    rng = np.random.default_rng(seed)
    kinds = ["plane", "sphere", "cylinder", "torus"]
    out = []
    for i in range(n):
        res = int(rng.integers(1, 22))
        F = int(rng.integers(2 if mode == "mi" else 1, 12))
        if mode == "mi":
            specs = [{"type": "sphere", "center": list(rng.uniform(-0.8, 0.8, 3)),
                      "radius": float(rng.uniform(0.0, 0.3))} for _ in range(F)]
        else:
            specs = [fns.random_function_spec(rng, kinds[int(rng.integers(0, 4))]) for _ in range(F)]
            if i % 3 == 0:
                # a plane through grid vertices and its duplicate: exact zeros, coincident planes
                xs = fns.grid_coords(res)[0]
                p = {"type": "plane", "point": [float(xs[res // 2]), 0.0, 0.0], "normal": [1.0, 0.0, 0.0]}
                specs += [p, dict(p)]
        lo = tuple(rng.uniform(-1.2, -0.8, 3)) if i % 4 == 1 else (-1.0, -1.0, -1.0)
        hi = tuple(rng.uniform(0.8, 1.2, 3)) if i % 4 == 1 else (1.0, 1.0, 1.0)
        out.append((res, fns.make_functions(specs), lo, hi))
    return out


def _check(pkg, probs, mode, **kw):
    batch = pkg.grid_batch(probs, mode=mode, **kw)
    assert len(batch) == len(probs)
    single = pkg.grid_implicit_arrangement if mode == "ia" else pkg.grid_material_interface
    for i, (res, funcs, lo, hi) in enumerate(probs):
        ref = single(res, funcs, bbox_min=lo, bbox_max=hi, **kw)
        view = batch.problem(i)
        for k in FIELDS:
            a, b = view[k], ref[k]
            assert a.shape == b.shape and np.array_equal(a, b), (i, k)
        st, rs = view.stats, ref.stats
        for k in STATS:
            assert st[k] == rs[k], (i, k)
        ref.close()
    batch.close()


@pytest.mark.parametrize("use_lookup", [True, False])
def test_batch_ia_equals_single_calls(pkg, fns, lib, use_lookup):
    _check(pkg, _problems(fns, 21, 14, "ia"), "ia", use_lookup=use_lookup)


def test_batch_mi_equals_single_calls(pkg, fns, lib):
    _check(pkg, _problems(fns, 22, 10, "mi"), "mi")


def test_batch_of_one_and_wide_functions(pkg, fns, lib):
    rng = np.random.default_rng(23)
    # 64 functions (the widest row), small spheres so that a tet holds few of them
    wide = fns.make_functions([{"type": "sphere", "center": list(rng.uniform(-0.9, 0.9, 3)),
                                "radius": float(rng.uniform(0.03, 0.12))} for _ in range(64)])
    narrow = fns.make_functions([fns.random_function_spec(rng, "plane")])
    _check(pkg, [(6, wide, (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0))], "ia")
    _check(pkg, [(3, narrow, (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)), (5, wide, (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)),
                 (2, narrow, (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0))], "ia")


def test_batch_workload_sample(pkg, fns, lib):
    """A slice of the batched benchmark workload (mixed kinds, 2..24 functions)."""
    wl = fns.workload_batch(n=24)
    _check(pkg, [(r, f, (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)) for r, f in wl.problems], "ia")


def test_batch_rejects_bad_problem(pkg, fns, lib):
    f = fns.make_functions([{"type": "zero"}])
    with pytest.raises(pkg.RiaError):
        pkg.grid_batch([(0, f)])
