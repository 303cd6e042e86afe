"""Exact rational brute force for one tet (test infrastructure).

An algorithm independent of the oracle's iterative cut: every vertex is found by solving all
independent 3-plane (IA) or 4-constraint (MI) systems in rational arithmetic, and the records are
checked for closure (faces on their planes, oriented as documented, cells tiling the tet).
Coordinates are barycentric (P0..P3); the reference frame for orientation is x = (P1, P2, P3).
"""
from fractions import Fraction as Fr
from itertools import combinations


def _rank(rows):
    m = [list(r) for r in rows]
    rank = 0
    ncol = len(m[0]) if m else 0
    for c in range(ncol):
        piv = None
        for r in range(rank, len(m)):
            if m[r][c] != 0:
                piv = r
                break
        if piv is None:
            continue
        m[rank], m[piv] = m[piv], m[rank]
        for r in range(len(m)):
            if r != rank and m[r][c] != 0:
                f = m[r][c] / m[rank][c]
                m[r] = [a - f * b for a, b in zip(m[r], m[rank])]
        rank += 1
    return rank


def _null_vector(rows, n):
    """One-dimensional null space of rows (len(rows) == n-1), or None."""
    m = [list(r) for r in rows]
    # Gaussian elimination to reduced row echelon form
    piv_cols = []
    rank = 0
    for c in range(n):
        piv = None
        for r in range(rank, len(m)):
            if m[r][c] != 0:
                piv = r
                break
        if piv is None:
            continue
        m[rank], m[piv] = m[piv], m[rank]
        pv = m[rank][c]
        m[rank] = [a / pv for a in m[rank]]
        for r in range(len(m)):
            if r != rank and m[r][c] != 0:
                f = m[r][c]
                m[r] = [a - f * b for a, b in zip(m[r], m[rank])]
        piv_cols.append(c)
        rank += 1
    if rank != n - 1:
        return None
    free = [c for c in range(n) if c not in piv_cols][0]
    v = [Fr(0)] * n
    v[free] = Fr(1)
    for r, c in enumerate(piv_cols):
        v[c] = -m[r][free]
    return v


def _greedy(labels, rowof, want):
    chosen = []
    for l in sorted(labels):
        if _rank([rowof(x) for x in chosen + [l]]) == len(chosen) + 1:
            chosen.append(l)
        if len(chosen) == want:
            break
    return tuple(chosen)


def _dot(a, b):
    return sum(x * y for x, y in zip(a, b))


def _grad(vals):
    return [vals[1] - vals[0], vals[2] - vals[0], vals[3] - vals[0]]


def _newell(pts):
    n = [Fr(0)] * 3
    for i in range(len(pts)):
        a, b = pts[i], pts[(i + 1) % len(pts)]
        n[0] += (a[1] - b[1]) * (a[2] + b[2])
        n[1] += (a[2] - b[2]) * (a[0] + b[0])
        n[2] += (a[0] - b[0]) * (a[1] + b[1])
    return n


def _xyz(P):
    return (P[1], P[2], P[3])


def _signed_volume(loops):
    """6 x signed volume enclosed by oriented (outward) polygon loops of reference coordinates."""
    vol = Fr(0)
    for loop in loops:
        p0 = loop[0]
        for i in range(1, len(loop) - 1):
            a, b = loop[i], loop[i + 1]
            vol += (p0[0] * (a[1] * b[2] - a[2] * b[1]) - p0[1] * (a[0] * b[2] - a[2] * b[0])
                    + p0[2] * (a[0] * b[1] - a[1] * b[0]))
    return vol


def ia_vertex_labels(planes):
    rows = {b: [Fr(int(b == c)) for c in range(4)] for b in range(4)}
    for i, p in enumerate(planes):
        rows[4 + i] = [Fr(x) for x in p]
    labels = list(rows)
    pts = {}
    for tri in combinations(labels, 3):
        n = _null_vector([rows[l] for l in tri], 4)
        if n is None:
            continue
        s = sum(n)
        if s == 0:
            continue
        P = tuple(x / s for x in n)
        if min(P) < 0:
            continue
        pts[P] = None
    out = {}
    for P in pts:
        tight = [l for l in labels if _dot(rows[l], P) == 0]
        out[_greedy(tight, lambda l: rows[l], 3)] = P
    return out, rows


def check_ia_record(planes, rec):
    """Assert that a decoded IA record is the arrangement of `planes` in canonical form."""
    expected, rows = ia_vertex_labels(planes)
    got = [tuple(v) for v in rec["verts"]]
    assert got == sorted(got), "vertices not sorted by label"
    assert set(got) == set(expected), (sorted(set(expected) - set(got)), sorted(set(got) - set(expected)))
    P = [expected[v] for v in got]
    edges = set()
    cell_loops = {}
    for f in rec["faces"]:
        loop = f["loop"]
        assert len(loop) >= 3 and loop[0] == min(loop)
        for v in loop:
            assert _dot(rows[f["supp"]], P[v]) == 0, "vertex off its face's plane"
        nrm = _newell([_xyz(P[v]) for v in loop])
        assert _dot(nrm, _grad(rows[f["supp"]])) > 0, "face not counter-clockwise seen from its positive side"
        for i in range(len(loop)):
            a, b = loop[i], loop[(i + 1) % len(loop)]
            edges.add((min(a, b), max(a, b)))
        pts = [_xyz(P[v]) for v in loop]
        cell_loops.setdefault(f["pos"], []).append(list(reversed(pts)))  # inward -> outward
        if f["neg"] is not None:
            cell_loops.setdefault(f["neg"], []).append(pts)
        assert f["boundary"] == (f["neg"] is None)
    nc = len(rec["cells"])
    assert sorted(cell_loops) == list(range(nc))
    total = Fr(0)
    for c in range(nc):
        v = _signed_volume(cell_loops[c])
        assert v > 0, "cell with non-positive volume"
        total += v
    assert total == 1, "cells do not tile the tet"
    assert len(got) - len(edges) + len(rec["faces"]) - nc == 1, "Euler characteristic"
    assert rec["cells"] == sorted(rec["cells"]) and len(set(rec["cells"])) == nc
    return True


def mi_vertex_labels(mats, owners=None):
    """Vertices of the material-interface complex.  `owners` (labels of the materials that own a
    cell) restricts the vertices to points fixed by the constraints of those materials; a material
    that only touches the maximum adds no geometry, but it still counts among the tied labels."""
    def row(l):
        if l < 4:
            return [Fr(int(l == c)) for c in range(4)] + [Fr(0)]
        return [Fr(x) for x in mats[l - 4]] + [Fr(-1)]

    labels = list(range(4 + len(mats)))
    pts = {}
    for quad in combinations(labels, 4):
        if all(l < 4 for l in quad):
            continue
        n = _null_vector([row(l) for l in quad], 5)
        if n is None:
            continue
        s = sum(n[:4])
        if s == 0:
            continue
        P = tuple(x / s for x in n[:4])
        t = n[4] / s
        if min(P) < 0:
            continue
        vals = [_dot([Fr(x) for x in m], P) for m in mats]
        if max(vals) != t:
            continue
        pts[P] = t
    out = {}
    for P, t in pts.items():
        tight = [b for b in range(4) if P[b] == 0]
        tight += [4 + i for i, m in enumerate(mats) if _dot([Fr(x) for x in m], P) == t]
        if owners is not None:
            own = [l for l in tight if l < 4 or l in owners]
            if not any(l >= 4 for l in own) or _rank([row(l) for l in own]) < 4:
                continue
        out[_greedy(tight, row, 4)] = P
    return out


def check_mi_record(mats, rec):
    expected = mi_vertex_labels(mats, owners=set(rec["cells"]))
    got = [tuple(v) for v in rec["verts"]]
    assert got == sorted(got)
    assert set(got) == set(expected), (sorted(set(expected) - set(got)), sorted(set(got) - set(expected)))
    P = [expected[v] for v in got]
    M = {4 + i: [Fr(x) for x in m] for i, m in enumerate(mats)}
    cell_loops = {}
    edges = set()
    keys = [(f["pos"], f["neg"]) for f in rec["faces"]]
    assert keys == sorted(keys) and len(set(keys)) == len(keys)
    for f in rec["faces"]:
        loop = f["loop"]
        assert len(loop) >= 3 and loop[0] == min(loop)
        pts = [_xyz(P[v]) for v in loop]
        nrm = _newell(pts)
        neg = f["neg"]
        for v in loop:
            mx = max(_dot(m, P[v]) for m in M.values())
            assert _dot(M[neg], P[v]) == mx
        if f["pos"] > 3:
            for v in loop:
                assert _dot(M[f["pos"]], P[v]) == _dot(M[neg], P[v])
            g = _grad([a - b for a, b in zip(M[f["pos"]], M[neg])])
            assert _dot(nrm, g) > 0
            cell_loops.setdefault(f["pos"], []).append(list(reversed(pts)))
        else:
            b = f["pos"]
            for v in loop:
                assert P[v][b] == 0
            g = _grad([Fr(int(b == c)) for c in range(4)])
            assert _dot(nrm, g) < 0, "boundary face not oriented out of the tet"
        cell_loops.setdefault(neg, []).append(pts)
        for i in range(len(loop)):
            a, c = loop[i], loop[(i + 1) % len(loop)]
            edges.add((min(a, c), max(a, c)))
    assert sorted(cell_loops) == sorted(rec["cells"])
    total = Fr(0)
    for c in rec["cells"]:
        v = _signed_volume(cell_loops[c])
        assert v > 0
        total += v
    assert total == 1
    assert len(got) - len(edges) + len(rec["faces"]) - len(rec["cells"]) == 1
    return True
