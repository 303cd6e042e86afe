"""The oracle's per-tet cut against an exact rational brute force (CPU only)."""
import numpy as np
import pytest

import bruteforce
from records import decode_ia, decode_mi


@pytest.fixture(autouse=True)
def _selfcheck(oracle):
    oracle.set_selfcheck(True)
    yield
    oracle.set_selfcheck(False)


def _ia(oracle, planes):
    rec = decode_ia(oracle.ia_cut(planes))
    bruteforce.check_ia_record(np.asarray(planes, dtype=np.float64).tolist(), rec)
    return rec


def _mi(oracle, mats):
    rec = decode_mi(oracle.mi_cut(mats))
    bruteforce.check_mi_record(np.asarray(mats, dtype=np.float64).tolist(), rec)
    return rec


def test_single_plane_corner(oracle):
    rec = _ia(oracle, [[-0.5, -0.5, -0.5, 0.5]])
    assert len(rec["verts"]) == 7 and len(rec["cells"]) == 2


@pytest.mark.parametrize("k", [1, 2, 3, 4])
def test_ia_random(oracle, k):
    rng = np.random.default_rng(100 + k)
    for _ in range(12 if k < 4 else 6):
        _ia(oracle, rng.normal(size=(k, 4)))


@pytest.mark.parametrize("k", [2, 3, 4])
def test_mi_random(oracle, k):
    rng = np.random.default_rng(200 + k)
    for _ in range(10):
        _mi(oracle, rng.normal(size=(k, 4)))


def test_ia_degenerate_planes(oracle):
    # plane through a tet corner, through an edge, coincident with a tet face, duplicated,
    # negated, the zero plane, and three planes through one interior line
    cases = [
        [[0.0, -1.0, 1.0, 0.5]],                       # through corner 0
        [[0.0, 0.0, 1.0, -1.0]],                       # through edge 0-1
        [[0.0, 0.0, 0.0, 2.0]],                        # the tet face opposite corner 3
        [[1.0, -2.0, 0.5, 0.25], [1.0, -2.0, 0.5, 0.25]],
        [[1.0, -2.0, 0.5, 0.25], [-2.0, 4.0, -1.0, -0.5]],
        [[0.0, 0.0, 0.0, 0.0], [1.0, -1.0, 1.0, -1.0]],
        [[1.0, -1.0, 0.0, 0.0], [0.0, 0.0, 1.0, -1.0], [1.0, -1.0, 1.0, -1.0]],
        [[1.0, -1.0, 0.0, 0.0], [0.0, 1.0, -1.0, 0.0], [1.0, 0.0, -1.0, 0.0], [0.0, 0.0, 1.0, -1.0]],
        [[0.0, 0.0, 1.0, -1.0], [0.0, 1.0, 0.0, -1.0], [0.0, 1.0, -1.0, 0.0]],
        [[0.0, 3.0, 0.0, 0.0], [1.0, -1.0, 1.0, -1.0]],  # coincident with face 1, plus a cut
    ]
    for planes in cases:
        _ia(oracle, planes)


def test_ia_degenerate_random_small_integers(oracle):
    # small integer values make exact zeros, shared lines and shared points frequent
    rng = np.random.default_rng(7)
    for _ in range(60):
        k = int(rng.integers(1, 5))
        _ia(oracle, rng.integers(-2, 3, size=(k, 4)).astype(np.float64))


def test_mi_degenerate_small_integers(oracle):
    """Integer materials: exact ties, identical materials, coincident tie planes, materials that
    touch the maximum without owning a cell."""
    rng = np.random.default_rng(8)
    for _ in range(150):
        k = int(rng.integers(2, 6))
        mats = rng.integers(-2, 3, size=(k, 4)).astype(np.float64)
        if rng.random() < 0.3:
            mats[-1] = mats[0]
        _mi(oracle, mats)


def test_mi_coincident_tie_planes(oracle):
    """m6 - m5 = 2 (m4 - m5) with material 4 owning no cell: the interface between 5 and 6 must be
    kept (it is labelled 4 by both clips)."""
    _mi(oracle, [[-1.0, 0.0, 0.0, 2.0], [-1.0, 2.0, -1.0, 2.0], [-1.0, -2.0, 1.0, 2.0], [-1.0, 2.0, -1.0, 2.0]])


def test_mi_duplicate_and_tie(oracle):
    _mi(oracle, [[1.0, 0.0, 0.0, 0.0], [1.0, 0.0, 0.0, 0.0], [0.0, 1.0, 0.0, 0.0]])
    _mi(oracle, [[1.0, 0.0, 0.0, 0.0], [0.0, 1.0, 0.0, 0.0], [0.0, 0.0, 1.0, 0.0], [0.0, 0.0, 0.0, 1.0]])
    _mi(oracle, [[0.5, 0.5, 0.0, 0.0], [0.0, 1.0, 0.0, 0.5]])


def test_reversed_order_is_consistent(oracle):
    """The reference's robustness mode (src/implicit_arrangement.cpp:137-243) re-runs every tet with
    the planes reversed and requires equal vertex/face/cell counts."""
    rng = np.random.default_rng(11)
    for _ in range(30):
        k = int(rng.integers(1, 5))
        p = rng.normal(size=(k, 4))
        a = decode_ia(oracle.ia_cut(p))
        b = decode_ia(oracle.ia_cut(p[::-1].copy()))
        assert (len(a["verts"]), len(a["faces"]), len(a["cells"])) == (len(b["verts"]), len(b["faces"]), len(b["cells"]))
        m = rng.normal(size=(k + 1, 4))
        a = decode_mi(oracle.mi_cut(m))
        b = decode_mi(oracle.mi_cut(m[::-1].copy()))
        assert (len(a["verts"]), len(a["faces"]), len(a["cells"])) == (len(b["verts"]), len(b["faces"]), len(b["cells"]))


def test_tiny_and_huge_magnitudes(oracle):
    _ia(oracle, [[1e-200, -1e-200, 3e-200, -2e-200], [1e150, -1e150, 2e150, -3e150]])
    _ia(oracle, [[1.0, -1.0, 1e-17, -1e-17], [1.0, -1.0, 2e-17, -1e-17]])
