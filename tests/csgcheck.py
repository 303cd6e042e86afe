"""CSG helpers for the tests: membership of a CSG tree, face labels by point evaluation, and the
reference's prune of patches, chains and corners (src/csg.cpp:55-116).

The point evaluation is independent of the library's labels: it evaluates the tree at two points
just off a face, on either side, from the linear interpolation of the function values over the
face's tet (the arrangement is that of the piecewise-linear functions).
"""
import numpy as np

INTER, UNION, NEG = 0, 1, 2


def inside(tree, vals, positive_inside=True):
    """Membership of a point with function values `vals` in the shape of `tree` (units [op, a, b]
    of a CSG tree file; None or empty: the union of all functions)."""
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


def face_label(f, xyz, face_offsets, face_verts, face_tets_first, face_func, pts, tets, fv, tree,
               positive_inside=True, eps=1e-7):
    """0 if the shape is on both sides of face f or on neither, 1 if it is on the positive side of
    the face's function, 2 if on the negative side; None where the evaluation is not conclusive
    (a degenerate polygon, or points too close to the face)."""
    P = xyz[face_verts[face_offsets[f]:face_offsets[f + 1]]]
    c = P.mean(axis=0)
    n = np.zeros(3)
    for i in range(len(P)):
        n += np.cross(P[i], P[(i + 1) % len(P)])
    if np.linalg.norm(n) < 1e-14:
        return None
    n /= np.linalg.norm(n)
    t = face_tets_first[f]
    T = pts[tets[t]]
    M = np.vstack([T.T, np.ones(4)])
    j = face_func[f][0]
    res = []
    for s in (eps, -eps):
        lam = np.linalg.solve(M, np.append(c + s * n, 1.0))
        vals = lam @ fv[tets[t]]
        res.append((vals[j], vals))
    (a, va), (b, vb) = res
    if min(abs(a), abs(b)) < 1e-12 or np.sign(a) == np.sign(b):
        return None
    vpos, vneg = (va, vb) if a > 0 else (vb, va)
    ip, ineg = inside(tree, vpos, positive_inside), inside(tree, vneg, positive_inside)
    return 0 if ip == ineg else (1 if ip else 2)


def patch_labels(patches, label_of_face):
    """A label per patch from the first face of it whose evaluation is conclusive (every face of a
    patch separates the same two cells)."""
    out = []
    for p in patches:
        lab = None
        for f in p:
            lab = label_of_face(f)
            if lab is not None:
                break
        assert lab is not None, "no face of the patch gave a conclusive label"
        out.append(lab)
    return out


def prune(patches, labels, face_vert_lists, n_verts, chains, edges, nm_degree):
    """src/csg.cpp:55-116: keep the patches whose two sides differ (label != 0), with the sign label
    of their positive side; keep the chains whose every edge has both ends counted at least twice
    in the faces of the kept patches; a vertex counted at most twice loses its non-manifold edges.
    Returns (kept patches, sign labels, kept chains, corners), corners being the vertices left with
    more than two non-manifold edges (the reference test's corners_count)."""
    kept, sign = [], []
    count = np.zeros(n_verts, dtype=np.int64)
    for p, lab in zip(patches, labels):
        if lab == 0:
            continue
        kept.append(list(p))
        sign.append(lab == 1)
        for f in p:
            for v in face_vert_lists[f]:
                count[v] += 1
    kept_chains = [list(c) for c in chains
                   if all(count[edges[e][0]] >= 2 and count[edges[e][1]] >= 2 for e in c)]
    nm = np.asarray(nm_degree).copy()
    nm[count <= 2] = 0
    return kept, sign, kept_chains, int((nm > 2).sum())


def nm_degree_from_faces(face_vert_lists, n_verts):
    """Non-manifold edges (more than two incident faces) per vertex, from the face vertex lists."""
    from collections import Counter

    count = Counter()
    for fl in face_vert_lists:
        for i in range(len(fl)):
            a, b = fl[i], fl[(i + 1) % len(fl)]
            count[(min(a, b), max(a, b))] += 1
    deg = np.zeros(n_verts, dtype=np.int64)
    for (a, b), c in count.items():
        if c > 2:
            deg[a] += 1
            deg[b] += 1
    return deg
