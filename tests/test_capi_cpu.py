"""CPU-only checks of the product library and of the device per-tet cut logic.

* libria.so loads and exports every function include/ria.h declares (no compute call: no GPU here).
* The device per-tet cut headers, compiled for the host by tests/hostcheck, reproduce the
  oracle's canonical records byte for byte (fast and exact variants).
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import REPO

sys.path.insert(0, os.path.join(REPO, "tests", "hostcheck"))


@pytest.fixture(scope="module")
def lib(pkg):
    pkg.build()
    return pkg.load()


def test_library_exports_every_declared_symbol(pkg, lib):
    names = pkg.declared_functions()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", pkg._lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert set(names) <= exported


def test_no_device_means_error_not_fallback(pkg, lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    assert lib.ria_device_count() == 0
    with pytest.raises(pkg.RiaError) as e:
        pkg.sample_functions(pkg.functions.make_functions([{"type": "zero"}]), np.zeros((1, 3)))
    assert e.value.status == pkg._lib.RIA_ENODEVICE


@pytest.fixture(scope="module")
def hc():
    import hc

    hc.lib()
    return hc


def _agree(hc, oracle, mode, rows):
    ref = oracle.ia_cut(rows) if mode == "ia" else oracle.mi_cut(rows)
    big, _ = hc.cut(mode, rows, True)
    assert big == ref
    fast, _ = hc.cut(mode, rows, False)
    assert isinstance(fast, int) or fast == ref
    return isinstance(fast, int)


def test_device_cut_logic_random(hc, oracle):
    rng = np.random.default_rng(5)
    for k in range(1, 7):
        for _ in range(60):
            _agree(hc, oracle, "ia", rng.normal(size=(k, 4)))
            _agree(hc, oracle, "mi", rng.normal(size=(k + 1, 4)))


def test_device_cut_logic_degenerate(hc, oracle):
    rng = np.random.default_rng(6)
    deferred = 0
    for _ in range(400):
        k = int(rng.integers(1, 5))
        deferred += _agree(hc, oracle, "ia", rng.integers(-2, 3, size=(k, 4)).astype(np.float64))
        k = int(rng.integers(2, 5))
        deferred += _agree(hc, oracle, "mi", rng.integers(-2, 3, size=(k, 4)).astype(np.float64))
    assert deferred > 0  # exact ties must reach the exact variant


def test_device_cut_logic_on_workload_tets(hc, oracle, fns):
    """Every active tet of the small implicit-arrangement workload and a slab of the material one."""
    for wl in (fns.workload_ia_small(res=10), fns.workload_mi(res=12)):
        pts, tets = fns.generate_tet_mesh(wl.res)
        fv = oracle.sample(wl.funcs, pts)
        r = oracle.run(wl.mode, pts, tets, fv)
        si, fit = r["start_index"], r["func_in_tet"]
        for t in range(len(tets)):
            if si[t + 1] == si[t]:
                continue
            rows = fv[tets[t]][:, fit[si[t]:si[t + 1]]].T.copy()
            ref = bytes(r["rec_bytes"][r["rec_offsets"][t]:r["rec_offsets"][t + 1]])
            got, _ = hc.cut(wl.mode, rows, True)
            assert got == ref, t


def test_exact_determinant_sign(hc):
    from fractions import Fraction

    rng = np.random.default_rng(9)
    for n in (2, 3, 4, 5):
        for _ in range(200):
            M = rng.integers(-3, 4, size=(n, n)).astype(np.float64) * 2.0 ** rng.integers(-60, 60, size=(n, n))
            if rng.random() < 0.3:
                M[-1] = M[0] * 2.0  # singular
            F = [[Fraction(float(x)) for x in row] for row in M]

            def det(m):
                if len(m) == 1:
                    return m[0][0]
                return sum((-1) ** c * m[0][c] * det([r[:c] + r[c + 1:] for r in m[1:]]) for c in range(len(m)))

            d = det(F)
            assert hc.det_sign(M) == (d > 0) - (d < 0)


def test_one_effective_plane_template_path(hc, oracle):
    """Tets whose planes reduce to one (duplicates, multiples, tet faces, zero planes) are built from
    the one-plane table; the record must equal the generic cut's."""
    rng = np.random.default_rng(12)
    seen = 0
    for _ in range(400):
        p = rng.integers(-2, 3, size=4).astype(np.float64)
        if rng.random() < 0.5:
            p = rng.normal(size=4)
        rows = [p]
        for _ in range(int(rng.integers(0, 4))):
            kind = rng.integers(0, 4)
            if kind == 0:
                rows.append(p * float(rng.choice([-2.0, 0.5, 1.0, 3.0])))
            elif kind == 1:
                b = np.zeros(4)
                b[int(rng.integers(0, 4))] = float(rng.choice([-1.5, 2.0]))
                rows.append(b)
            elif kind == 2:
                rows.append(np.zeros(4))
            else:
                rows.append(p.copy())
        rng.shuffle(rows)
        rows = np.array(rows)
        got = hc.ia_template(rows)
        if got is None:
            continue
        seen += 1
        assert got[0] == oracle.ia_cut(rows)
        big, summ = hc.cut("ia", rows, True)
        assert got[0] == big and np.array_equal(got[1], summ[:4])
    assert seen > 300
