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


def test_tuning_records_do_not_change_results(pkg, fns, lib):
    """Every tuning record (the heavy/light split, the warp-cut bin size, resident blocks, the thread
    kernel's block, the cut stage as a CUDA graph or not, on batches and on single calls) gives the same
    fields, bit for bit."""
    probs = _problems(fns, 91, 24, "ia")
    wl = fns.workload_ia_degenerate(res=40)
    start = pkg.get_tuning()
    try:
        ref_batch = pkg.grid_batch(probs)
        ref_single = pkg.grid_implicit_arrangement(wl.res, wl.funcs)
        for rec in ({"warp_route": 64, "warp_blocks_per_sm": 1, "fast_block": 32, "cut_graph": 2, "heavy_min_k": 3},
                    {"warp_route": 0, "warp_blocks_per_sm": 2, "fast_block": 64, "cut_graph": 0, "heavy_min_k": 8},
                    {"warp_route": 1 << 20, "warp_blocks_per_sm": 0, "fast_block": 128, "cut_graph": 1,
                     "heavy_min_k": 0}):
            pkg.set_tuning(dict(start, **rec))
            got = pkg.grid_batch(probs)
            for i in range(len(probs)):
                for k in FIELDS:
                    assert np.array_equal(got.problem(i)[k], ref_batch.problem(i)[k]), (rec, i, k)
            got.close()
            single = pkg.grid_implicit_arrangement(wl.res, wl.funcs)
            for k in FIELDS:
                assert np.array_equal(single[k], ref_single[k]), (rec, k)
            single.close()
    finally:
        pkg.set_tuning(start)


def test_mi_tuning_records_do_not_change_results(pkg, fns, lib):
    """The material interface's heavy/light split (its heavy bins from three, four, five or eight
    materials up) and the launch shapes give the same fields, bit for bit, on batches and single calls."""
    probs = _problems(fns, 93, 16, "mi")
    wl = fns.workload_mi(res=24)
    start = pkg.get_tuning()
    assert start["mi_heavy_min_k"] in (0, 3, 4, 5)
    try:
        ref_batch = pkg.grid_batch(probs, mode="mi")
        ref_single = pkg.grid_material_interface(wl.res, wl.funcs)
        for rec in ({"mi_heavy_min_k": 3, "fast_block": 32, "cut_graph": 2}, {"mi_heavy_min_k": 5, "cut_graph": 0},
                    {"mi_heavy_min_k": 8, "fast_block": 128}, {"mi_heavy_min_k": 0}):
            pkg.set_tuning(dict(start, **rec))
            got = pkg.grid_batch(probs, mode="mi")
            for i in range(len(probs)):
                for k in FIELDS:
                    assert np.array_equal(got.problem(i)[k], ref_batch.problem(i)[k]), (rec, i, k)
            got.close()
            single = pkg.grid_material_interface(wl.res, wl.funcs)
            for k in FIELDS:
                assert np.array_equal(single[k], ref_single[k]), (rec, k)
            single.close()
    finally:
        pkg.set_tuning(start)


def test_autotune_installs_a_record(pkg, fns, lib):
    """The autotuner times its candidate records on a sample and installs the fastest, which is never
    slower than the record it started from (that record is among the timed ones)."""
    start = pkg.get_tuning()
    try:
        probs = _problems(fns, 92, 32, "ia")
        best, best_s, default_s = pkg.autotune(probs, reps=1)
        assert best == pkg.get_tuning()
        assert 0 < best_s <= default_s
        assert best["fast_block"] in (0, 32, 64, 128) and best["cut_graph"] in (0, 1, 2)
        assert best["heavy_min_k"] in (0, 3, 4, 5, 6)
    finally:
        pkg.set_tuning(start)


def test_bad_tuning_rejected(pkg, lib):
    start = pkg.get_tuning()
    for bad in ({"fast_block": 48}, {"cut_graph": 3}, {"warp_route": -1}, {"heavy_min_k": 2}, {"mi_heavy_min_k": 9}):
        with pytest.raises(pkg.RiaError):
            pkg.set_tuning(dict(start, **bad))
    assert pkg.get_tuning() == start
