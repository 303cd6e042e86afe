"""CSG pruning on the device (ria_mesh_csg / ria_batch_csg, src/csg.cpp:55-116) against an independent
geometric check: the CSG membership is evaluated at two points just off each face, from the linear
interpolation of the function values in the face's tet."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INTER, UNION, NEG = 0, 1, 2


def _inside(tree, vals, positive_inside=True):
    ins = vals > 0 if positive_inside else vals < 0
    if not tree:
        return bool(ins.any())

    def ev(e):
        if e < 0:
            return bool(ins[-e - 1])
        op, a, b = tree[e - 1]
        if op == NEG:
            return not ev(a)
        return (ev(a) and ev(b)) if op == INTER else (ev(a) or ev(b))
    return ev(1)


def _geometric_labels(mesh, pts, tets, fv, tree, positive_inside=True):
    """Label of each face from point evaluations; None where the check is not conclusive."""
    xyz, fo, fvs = mesh["xyz"], mesh["face_offsets"], mesh["face_verts"]
    fto, ftets, ffunc = mesh["face_tet_offsets"], mesh["face_tets"], mesh["face_func"]
    out = []
    for f in range(len(fo) - 1):
        P = xyz[fvs[fo[f]:fo[f + 1]]]
        c = P.mean(axis=0)
        n = np.zeros(3)
        for i in range(len(P)):
            n += np.cross(P[i], P[(i + 1) % len(P)])
        if np.linalg.norm(n) < 1e-14:
            out.append(None)
            continue
        n /= np.linalg.norm(n)
        t = ftets[fto[f]][0]
        T = pts[tets[t]]
        M = np.vstack([T.T, np.ones(4)])
        j = ffunc[f][0]
        res = []
        for s in (1e-7, -1e-7):
            lam = np.linalg.solve(M, np.append(c + s * n, 1.0))
            vals = lam @ fv[tets[t]]
            res.append((vals[j], vals))
        (a, va), (b, vb) = res
        if min(abs(a), abs(b)) < 1e-12 or np.sign(a) == np.sign(b):
            out.append(None)
            continue
        vpos, vneg = (va, vb) if a > 0 else (vb, va)
        ip, ineg = _inside(tree, vpos, positive_inside), _inside(tree, vneg, positive_inside)
        out.append(0 if ip == ineg else (1 if ip else 2))
    return out


def _shapes(fns, seed, n):
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n):
        if i % 2:
            specs.append({"type": "sphere", "center": list(rng.uniform(-0.5, 0.5, 3)),
                          "radius": float(rng.uniform(0.25, 0.55))})
        else:
            specs.append({"type": "cylinder", "axis_point": list(rng.uniform(-0.3, 0.3, 3)),
                          "axis_vector": list(rng.normal(size=3)), "radius": float(rng.uniform(0.15, 0.35))})
    return fns.make_functions(specs)


TREES = [
    None,                                                 # union of all (the reference's default)
    [(INTER, -1, -2)],
    [(UNION, 2, -3), (INTER, -1, -2)],                    # (f0 & f1) | f2
    [(INTER, -1, 2), (NEG, -2, 0)],                       # f0 minus f1
    [(UNION, 2, 3), (INTER, -1, 4), (INTER, -3, -4), (NEG, -2, 0)],  # (f0 - f1) | (f2 & f3)
]


@pytest.mark.parametrize("ti", range(len(TREES)))
def test_csg_labels_match_point_evaluation(pkg, fns, ti):
    pkg.build()
    funcs = _shapes(fns, 30 + ti, 4)
    res = 18
    mesh = pkg.grid_implicit_arrangement(res, funcs)
    pts, tets = fns.generate_tet_mesh(res)
    fv = mesh["func_vals"].reshape(len(pts), len(funcs))
    for pos in (True, False):
        got = mesh.csg(TREES[ti], positive_inside=pos)
        ref = _geometric_labels(mesh, pts, tets, fv, TREES[ti], pos)
        checked = [(g, r) for g, r in zip(got.tolist(), ref) if r is not None]
        assert len(checked) > 0.95 * len(ref)
        assert all(g == r for g, r in checked)
        assert 0 < int((got > 0).sum()) < len(got) or ti == 0


def test_csg_in_a_batch_equals_single(pkg, fns):
    pkg.build()
    probs = [(12 + i, _shapes(fns, 40 + i, 3 + i % 2)) for i in range(4)]
    batch = pkg.grid_batch(probs)
    tree = [(UNION, 2, -3), (INTER, -1, -2)]
    for i, (r, f) in enumerate(probs):
        single = pkg.grid_implicit_arrangement(r, f)
        assert np.array_equal(batch.problem(i).csg(tree), single.csg(tree))
        assert np.array_equal(batch.problem(i).csg(None, positive_inside=False), single.csg(None, positive_inside=False))


def test_csg_rejects_bad_trees(pkg, fns):
    pkg.build()
    mesh = pkg.grid_implicit_arrangement(6, _shapes(fns, 50, 2))
    for bad in ([(INTER, -1, -3)], [(UNION, 2, -1)], [(7, -1, -2)], [(INTER, 1, -1)]):
        with pytest.raises(pkg.RiaError):
            mesh.csg(bad)


def test_face_sides_agree_with_labels(pkg, fns):
    """The two side sign vectors reproduce the device tree evaluation for any membership function."""
    pkg.build()
    funcs = _shapes(fns, 60, 4)
    mesh = pkg.grid_implicit_arrangement(14, funcs)
    sides = mesh.face_sides()
    tree = TREES[4]
    labels = mesh.csg(tree)
    for f, (sp, sn) in enumerate(sides.tolist()):
        vp = np.array([1.0 if (sp >> j) & 1 else -1.0 for j in range(len(funcs))])
        vn = np.array([1.0 if (sn >> j) & 1 else -1.0 for j in range(len(funcs))])
        ip, ineg = _inside(tree, vp), _inside(tree, vn)
        assert labels[f] == (0 if ip == ineg else (1 if ip else 2))
