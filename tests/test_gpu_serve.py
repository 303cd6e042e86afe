"""The served form (ria_server_*): a mixed stream of arrangement, material-interface and CSG
requests, submitted while earlier ones are on the GPU; every result equals the same request alone
(its plain grid call, and ria_mesh_csg for CSG)."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("xyz", "verts", "face_offsets", "face_verts", "face_tets", "face_func", "func_vals")
TREES = [None, [(0, -1, -2)], [(1, 2, -3), (0, -1, -2)], [(0, -1, 2), (2, -2, 0)]]


def _request(fns, rng, i):
    kind = ["ia", "ia", "ia", "mi", "mi", "csg"][i % 6]
    res = int(rng.integers(6, 26))
    F = int(rng.integers(3, 9))
    if kind == "mi":
        specs = [{"type": "sphere", "center": list(rng.uniform(-0.8, 0.8, 3)), "radius": float(rng.uniform(0, 0.3))}
                 for _ in range(F)]
    elif kind == "csg":
        specs = [fns.random_function_spec(rng, ["sphere", "cylinder"][j % 2]) for j in range(F)]
    else:
        specs = [fns.random_function_spec(rng, ["plane", "sphere", "cylinder", "torus"][j % 4]) for j in range(F)]
    tree = TREES[i % len(TREES)] if kind == "csg" else None
    return kind, res, fns.make_functions(specs), tree


def _alone(pkg, kind, res, funcs, tree):
    m = (pkg.grid_material_interface if kind == "mi" else pkg.grid_implicit_arrangement)(res, funcs)
    return m, (m.csg(tree) if kind == "csg" else None)


def test_mixed_stream_equals_alone(pkg, fns):
    pkg.build()
    rng = np.random.default_rng(70)
    reqs = [_request(fns, rng, i) for i in range(48)]
    srv = pkg.Server(budget_bytes=4 << 30, streams=3, max_batch=16)
    tickets = [None] * len(reqs)

    def producer():  # requests arrive while earlier ones run
        for i, (kind, res, funcs, tree) in enumerate(reqs):
            tickets[i] = srv.submit(kind, res, funcs, tree=tree)
            time.sleep(0.002 * (i % 4))
    th = threading.Thread(target=producer)
    th.start()
    th.join()
    lat = []
    for i, (kind, res, funcs, tree) in enumerate(reqs):
        view, latency = srv.wait(tickets[i], timeout=300.0)
        lat.append(latency)
        ref, ref_labels = _alone(pkg, kind, res, funcs, tree)
        for k in FIELDS:
            a, b = view[k], ref[k]
            a = a.reshape(b.shape) if a.size == b.size else a
            assert a.shape == b.shape and np.array_equal(a, b), (i, kind, k)
        if kind == "csg":
            assert np.array_equal(srv.labels(tickets[i]), ref_labels), i
        ref.close()
        srv.release(tickets[i])
    assert all(x > 0 for x in lat)
    srv.close()


def test_budget_and_timeouts(pkg, fns):
    pkg.build()
    f = fns.make_functions([{"type": "sphere", "center": [0, 0, 0], "radius": 0.5}])
    srv = pkg.Server(budget_bytes=64 << 20, streams=1)
    with pytest.raises(pkg.RiaError):
        srv.submit("ia", 400, f)  # larger than the whole budget
    t = srv.submit("ia", 8, f)
    view, _ = srv.wait(t, timeout=120.0)
    assert view.stats["num_faces"] > 0
    with pytest.raises(pkg.RiaError):
        srv.wait(12345, timeout=0.0)
    srv.release(t)
    srv.close()
