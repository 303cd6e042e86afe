"""The oracle's local-to-global maps (the reference's extraction variants, src/extract_mesh.cpp:268-566
and 988-1443) against the mesh they index, on the CPU: every record vertex of a face listed for a
tet maps to that face's mesh vertex (or to the tet vertex it lies on, as -v-1), and every occurrence
the mesh lists is named in the face map."""
import numpy as np
import pytest

from records import decode_ia, decode_mi, split_records


def _check(mode, r, tets):
    verts, fo, fv = r["verts"], r["face_offsets"], r["face_verts"]
    vo, tv, fo2, tf = r["tet_vert_offsets"], r["tet_verts"], r["tet_face_offsets"], r["tet_faces"]
    recs = split_records(r["rec_offsets"], r["rec_bytes"])
    assert len(vo) == len(fo2) == len(tets) + 1
    assert not (tv == np.iinfo(np.int64).min).any()
    seen = np.zeros(len(fo) - 1, dtype=np.int64)
    for t, b in enumerate(recs):
        if b is None:
            assert vo[t + 1] == vo[t] and fo2[t + 1] == fo2[t]
            continue
        rec = decode_ia(b) if mode == "ia" else decode_mi(b)
        vmap = tv[vo[t]:vo[t + 1]]
        fmap = tf[fo2[t]:fo2[t + 1]]
        assert len(vmap) == len(rec["verts"]) and len(fmap) == len(rec["faces"])
        for j, g in enumerate(vmap):
            if g < 0:
                assert -g - 1 in tets[t]
        for j, face in enumerate(rec["faces"]):
            f = fmap[j]
            if f < 0:
                continue
            seen[f] += 1
            # the same vertices (another occurrence of a face on the tet boundary runs its loop from
            # another start and the other way round); a record vertex on a tet vertex maps to -v-1,
            # where the mesh names the vertex record on that tet vertex
            want = fv[fo[f]:fo[f + 1]]
            named = [int(w) if verts[w][2] != 1 else -int(verts[w][3]) - 1 for w in want]
            assert sorted(vmap[face["loop"]].tolist()) == sorted(named)
    # every occurrence the mesh lists is named, and nothing else
    fto, ftt = r["face_tet_offsets"], r["face_tets"]
    for f in range(len(fo) - 1):
        for e in range(fto[f], fto[f + 1]):
            t, j = ftt[e]
            assert tf[fo2[t] + j] == f
    if mode == "ia":
        assert np.array_equal(seen, np.diff(fto))


@pytest.mark.parametrize("mode", ["ia", "mi"])
def test_maps_match_the_mesh(mode, fns, oracle):
    wl = fns.workload_ia_degenerate(res=10) if mode == "ia" else fns.workload_mi(res=10)
    pts, tets = fns.generate_tet_mesh(wl.res)
    r = oracle.run(mode, pts, tets, oracle.sample(wl.funcs, pts))
    _check(mode, r, tets)


def test_maps_boundary_interfaces(fns, oracle):
    """Integer materials with exact ties: material-interface faces on the tet boundary, named in both
    tets that share them (src/extract_mesh.cpp:1431)."""
    rng = np.random.default_rng(4)
    pts, tets = fns.generate_tet_mesh(6)
    both = 0
    for _ in range(5):
        fv = rng.integers(-2, 3, size=(len(pts), 4)).astype(np.float64)
        fv[:, 3] = fv[:, 1]
        r = oracle.run("mi", pts, tets, fv)
        _check("mi", r, tets)
        tf = r["tet_faces"]
        both += int((np.bincount(tf[tf >= 0]) == 2).sum())
    assert both > 0
