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
from records import decode_ia, decode_mi

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
    big, bsum = hc.cut(mode, rows, True)
    assert big == ref
    fast, _ = hc.cut(mode, rows, False)
    assert isinstance(fast, int) or fast == ref
    mid, _ = hc.cut(mode, rows, "mid")
    assert isinstance(mid, int) or mid == ref
    if mode == "ia":
        warp, wsum = hc.cut(mode, rows, "warp")
        assert warp == ref and np.array_equal(wsum[:4], bsum[:4])
        light, lsum = hc.cut(mode, rows, "warp_light")  # may report its smaller capacity
        assert light in (-11, -10 - 1) or (light == ref and np.array_equal(lsum[:4], bsum[:4]))
    else:
        split, ssum = hc.cut(mode, rows, "warp")  # the material interface's split path
        assert isinstance(split, int) or (split == ref and np.array_equal(ssum[:5], bsum[:5]))
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


def test_device_cut_near_degenerate(hc, oracle):
    """Exact degeneracies perturbed at and below FP32 resolution (2^-24 relative): the FP32 filter
    must hand these predicates on to the FP64 filter or the exact evaluation, never decide them."""
    rng = np.random.default_rng(10)
    for _ in range(300):
        k = int(rng.integers(1, 5))
        base = rng.integers(-2, 3, size=(k, 4)).astype(np.float64)
        eps = 10.0 ** rng.uniform(-9, -5, size=(k, 4)) * rng.choice([-1.0, 0.0, 1.0], size=(k, 4))
        _agree(hc, oracle, "ia", base + eps)
        base = rng.integers(-2, 3, size=(k + 1, 4)).astype(np.float64)
        eps = 10.0 ** rng.uniform(-9, -5, size=(k + 1, 4)) * rng.choice([-1.0, 0.0, 1.0], size=(k + 1, 4))
        _agree(hc, oracle, "mi", base + eps)


def test_device_mi_dominated_materials(hc, oracle):
    """Materials below another at every corner (strictly, or with ties at some corners) are skipped by
    the device cut; the records must still equal the oracle's full clipping."""
    rng = np.random.default_rng(9)
    for _ in range(200):
        k = int(rng.integers(3, 7))
        m = rng.integers(-3, 4, size=(k, 4)).astype(np.float64)
        a, b = rng.choice(k, size=2, replace=False)
        m[a] = m[b] - rng.integers(0, 2, size=4)  # a <= b everywhere, strict where 1
        if rng.random() < 0.5:
            m[a] = m[b] - 1.0 - rng.random(4)      # strictly below
        _agree(hc, oracle, "mi", m)


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


def test_two_group_template_path(hc, oracle):
    """Tets whose planes reduce to two groups (duplicates, multiples, tet faces, zero planes besides two
    distinct planes) take the two representatives' record, relabelled; it must equal the generic cut's."""
    rng = np.random.default_rng(13)
    seen = 0
    for _ in range(400):
        base = []
        for _ in range(2):
            p = rng.integers(-2, 3, size=4).astype(np.float64)
            if rng.random() < 0.5:
                p = rng.normal(size=4)
            base.append(p)
        rows = list(base)
        for _ in range(int(rng.integers(0, 5))):
            kind = rng.integers(0, 4)
            p = base[int(rng.integers(0, 2))]
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
        got = hc.ia_template2(rows)
        if got is None:
            continue
        seen += 1
        assert got[0] == oracle.ia_cut(rows)
        big, summ = hc.cut("ia", rows, True)
        assert got[0] == big and np.array_equal(got[1], summ[:4])
    assert seen > 250


def _exact_key(mode, rows):
    """The secondary-lookup key restated with rational arithmetic."""
    from fractions import Fraction as Fr
    from itertools import combinations

    def sgn(x):
        return (x > 0) - (x < 0)
    R = [[Fr(x) for x in r] for r in np.asarray(rows, dtype=np.float64)]
    t = []
    if mode == "ia":
        P, Q = R
        t = [sgn(x) for x in P] + [sgn(x) for x in Q]
        t += [sgn(P[i] * Q[j] - P[j] * Q[i]) for i, j in combinations(range(4), 2)]
    else:
        for a, b in ((0, 1), (0, 2), (1, 2)):
            t += [sgn(R[b][c] - R[a][c]) for c in range(4)]
        t += [sgn((R[1][c] - R[0][c]) * (R[2][d] - R[0][d]) - (R[2][c] - R[0][c]) * (R[1][d] - R[0][d]))
              for c, d in combinations(range(4), 2)]
    k = 0
    for s in t:
        k = 3 * k + s + 1
    return k


def test_secondary_lookup_keys(hc, oracle):
    """The device keys equal their rational restatement, and equal keys always carry equal records
    (the combinatorial type fixes the canonical record), for generic and degenerate inputs."""
    rng = np.random.default_rng(12)
    seen = {}
    for it in range(8000):
        mode = "ia" if it % 2 == 0 else "mi"
        n = 2 if mode == "ia" else 3
        kind = (it // 2) % 4
        if kind == 0:
            rows = rng.normal(size=(n, 4))
        elif kind == 1:
            rows = rng.integers(-2, 3, size=(n, 4)).astype(np.float64)
        elif kind == 2:
            rows = rng.integers(-1, 2, size=(n, 4)).astype(np.float64) + rng.normal(size=(n, 4)) * 1e-9
        else:  # the seeding's random rows: exact zeros among values of mixed magnitudes
            rows = rng.normal(size=(n, 4)) * np.exp2(rng.integers(-4, 4, size=(n, 4)))
            rows[rng.random((n, 4)) < 0.125] = 0.0
        k = hc.key(mode, rows)
        assert k == _exact_key(mode, rows)
        rec = oracle.ia_cut(rows) if mode == "ia" else oracle.mi_cut(rows)
        d = decode_ia(rec) if mode == "ia" else decode_mi(rec)
        if d["rep"] != list(range(4, 4 + n)):
            continue
        assert seen.setdefault((mode, k), rec) == rec
    assert hc.key("ia", [[1e-80, 1, 1, 1], [1, 2, 3, 4]]) is None


def test_heavy_tets_exact_variant(hc, oracle):
    """Up to 14 planes (more than 256 faces) and 16 materials in one tet: the exact variant either
    reports its capacity or reproduces the oracle's record."""
    rng = np.random.default_rng(13)
    done = 0
    for k in (10, 12, 14):
        for _ in range(6):
            rows = rng.normal(size=(k, 4))
            out, _ = hc.cut("ia", rows, True)
            if not isinstance(out, int):
                assert out == oracle.ia_cut(rows)
                done += 1
    for k in (8, 12, 16):
        for _ in range(4):
            rows = rng.normal(size=(k, 4)) * 0.3
            out, _ = hc.cut("mi", rows, True)
            assert not isinstance(out, int) and out == oracle.mi_cut(rows)
    assert done >= 8


def test_warp_variant_heavy_and_degenerate(hc, oracle):
    """The warp variant (its lane-parallel steps run serially here) on the heavy bins it serves:
    four to ten planes, random, integer-degenerate and with duplicated planes.  It either reports
    its capacity or reproduces the oracle's record and summary."""
    rng = np.random.default_rng(14)
    done = 0
    for k in range(4, 11):
        for trial in range(30):
            if trial % 3 == 0:
                rows = rng.normal(size=(k, 4))
            elif trial % 3 == 1:
                rows = rng.integers(-2, 3, size=(k, 4)).astype(np.float64)
            else:
                base = rng.normal(size=(max(2, k // 2), 4))
                rows = np.array([base[int(rng.integers(0, len(base)))] * float(rng.choice([1.0, -2.0, 0.5]))
                                 for _ in range(k)])
            out, summ = hc.cut("ia", rows, "warp")
            if isinstance(out, int):
                assert out == -11  # capacity
                continue
            big, bsum = hc.cut("ia", rows, True)
            assert out == oracle.ia_cut(rows) == big and np.array_equal(summ[:4], bsum[:4])
            done += 1
    assert done >= 150


def test_warp_light_state_on_light_bins(hc, oracle, fns):
    """The warp variant's light state (three quarters of the vertex and face room) on the tets it
    serves: the light bins' leftovers of the large degenerate workload (three to five active
    functions) and random three- to five-plane tets.  It reproduces the oracle's record, or reports its capacity (the full
    warp state then takes the tet); most of these tets fit."""
    wl = fns.workload_ia_degenerate(res=12)
    pts, tets = fns.generate_tet_mesh(wl.res)
    fv = oracle.sample(wl.funcs, pts)
    r = oracle.run("ia", pts, tets, fv)
    si, fit = r["start_index"], r["func_in_tet"]
    rows_list = []
    for t in range(len(tets)):
        k = si[t + 1] - si[t]
        if 3 <= k <= 5:
            rows_list.append(fv[tets[t]][:, fit[si[t]:si[t + 1]]].T.copy())
    rng = np.random.default_rng(41)
    for k in (3, 4, 5):
        rows_list += [rng.normal(size=(k, 4)) for _ in range(40)]
    fits = 0
    for rows in rows_list:
        out, summ = hc.cut("ia", rows, "warp_light")
        if isinstance(out, int):
            assert out in (-11, -10 - 1)  # capacity (CUT_DEFER)
            continue
        big, bsum = hc.cut("ia", rows, True)
        assert out == oracle.ia_cut(rows) == big and np.array_equal(summ[:4], bsum[:4])
        fits += 1
    assert len(rows_list) > 150 and fits >= 0.8 * len(rows_list), (fits, len(rows_list))


def test_split_variant_heavy_and_degenerate(hc, oracle):
    """The material interface's warp variant (per-lane clips, then the lane-parallel merge; its
    lane-parallel steps run serially here) on the heavy bins it serves: four to 32 materials, random,
    integer-degenerate (ties and dominated materials) and with duplicated materials.  It either
    defers the tet or reproduces the oracle's record and the exact variant's summary.  Exact ties
    defer (its predicates are filtered), and so do cells beyond its capacities, which random tets
    with twelve or more materials reach; up to eight materials every tie-free tet completes."""
    rng = np.random.default_rng(15)
    done = 0
    for k in (4, 5, 6, 8, 12, 16, 24, 32):
        for trial in range(12):
            if trial % 3 == 0:
                rows = rng.normal(size=(k, 4)) * 0.3
            elif trial % 3 == 1:
                rows = rng.integers(-2, 3, size=(k, 4)).astype(np.float64)
            else:
                base = rng.normal(size=(max(2, k // 2), 4)) * 0.3
                rows = np.array([base[int(rng.integers(0, len(base)))] for _ in range(k)])
            out, summ = hc.cut("mi", rows, "warp")
            if isinstance(out, int):
                assert out == -11  # deferred
                assert k > 8 or trial % 3 == 1
                continue
            big, bsum = hc.cut("mi", rows, True)
            assert out == oracle.mi_cut(rows) == big and np.array_equal(summ[:5], bsum[:5])
            done += 1
    assert done >= 50


def test_sampler_square_root_is_correctly_rounded(hc):
    """The sampler's integer square root (sqrt_rn.cuh) against the C library's correctly rounded
    sqrt, bit for bit: random bit patterns over the whole double range (negative, subnormal,
    infinite and NaN inputs included), mantissas at both ends of every binade tested, perfect
    squares and their neighbours.  The same inputs with the seed moved by 2^-20 (relative), about
    four times the FP32 reciprocal square root's documented error, must still round correctly."""
    rng = np.random.default_rng(16)
    vals = [rng.integers(0, 2**64 - 1, size=400_000, dtype=np.uint64).view(np.float64),
            rng.integers(0, 2**63, size=400_000, dtype=np.uint64).view(np.float64),
            rng.uniform(0, 10, size=400_000) ** rng.uniform(-3, 3, size=400_000)]
    for e in (1, 1023 - 52, 1022, 1023, 1024, 2045, 2046):
        base = np.uint64(e) << np.uint64(52)
        steps = np.arange(20_000, dtype=np.uint64)
        vals.append((base + steps).view(np.float64))
        vals.append((base + (np.uint64(1) << np.uint64(52)) - np.uint64(1) - steps).view(np.float64))
    k = rng.integers(1, 2**26, size=200_000).astype(np.float64)
    sq = k * k
    vals += [sq, np.nextafter(sq, 0), np.nextafter(sq, np.inf)]
    vals.append(np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, 2.2250738585072014e-308,
                          1.7976931348623157e308, 0.25, 1.0, 2.0, 4.0]))
    v = np.concatenate(vals)
    with np.errstate(invalid="ignore"):
        ref = np.sqrt(v)
    for perturb in (0, -1, 1):
        out = hc.sqrt_rn(v, perturb)
        same = (out.view(np.uint64) == ref.view(np.uint64)) | (np.isnan(out) & np.isnan(ref))
        assert same.all(), (perturb, v[~same][:4])


def test_vertex_division_is_correctly_rounded(hc):
    """The vertex emission's division (div_rn.cuh: reciprocal by Newton steps in integer arithmetic,
    finished from the exact remainder) against IEEE 754 division (numpy), bit for bit: random bit
    patterns over the whole range (zero, subnormal, infinite and NaN operands and out-of-range
    quotients go to the FP64 instruction), normal operands of every significand and nearby exponents,
    divisors at both ends of a binade (the reciprocal seed's extremes), exact quotients and quotients
    one unit off them (a quotient of two doubles is never halfway between two doubles, so these are
    the cases that test the remainder's fix-up), and the emission's own operands f2 / (f2 - f1)."""
    rng = np.random.default_rng(29)
    n = 400_000

    def bits(lo, hi, size):
        return rng.integers(lo, hi, size=size, dtype=np.uint64).view(np.float64)

    pairs = [(bits(0, 2**64 - 1, n), bits(0, 2**64 - 1, n))]
    e = rng.integers(1000, 1050, size=n).astype(np.uint64)
    fa = rng.integers(0, 2**52, size=n, dtype=np.uint64)
    fb = rng.integers(0, 2**52, size=n, dtype=np.uint64)
    sa = rng.integers(0, 2, size=n).astype(np.uint64) << np.uint64(63)
    a = (sa | (e << np.uint64(52)) | fa).view(np.float64)
    b = ((rng.integers(1000, 1050, size=n).astype(np.uint64) << np.uint64(52)) | fb).view(np.float64)
    pairs.append((a, b))
    # divisors at the ends of a binade, and just inside them
    for fr in (0, 1, 2**29 - 1, 2**29, 2**52 - 1, 2**52 - 2**29, 2**52 - 2):
        bb = ((rng.integers(1000, 1050, size=n // 8).astype(np.uint64) << np.uint64(52)) | np.uint64(fr)).view(np.float64)
        pairs.append((a[: n // 8], bb))
    # exact quotients, and one unit off: q * b with integer-like q
    q = rng.integers(1, 2**26, size=n).astype(np.float64)
    bq = rng.uniform(0.5, 2.0, size=n)
    prod = q * bq
    pairs += [(prod, bq), (np.nextafter(prod, np.inf), bq), (np.nextafter(prod, 0), bq)]
    # exact quotients of odd significands
    odd = (rng.integers(2**52, 2**53, size=n, dtype=np.uint64) | np.uint64(1)).astype(np.float64)
    pairs += [(odd, np.full(n, 2.0)), (odd * 3.0, np.full(n, 6.0)), (odd, np.full(n, 0.25))]
    # the emission's operands: values of a function at two corners across a crossing
    f1 = rng.uniform(-1, 1, n) * 10.0 ** rng.uniform(-12, 2, n)
    f2 = -np.sign(f1) * rng.uniform(0, 1, n) * 10.0 ** rng.uniform(-12, 2, n)
    with np.errstate(all="ignore"):
        pairs.append((f2, f2 - f1))
    pairs.append((np.array([0.0, -0.0, 1.0, 1.0, np.inf, 1.0, np.nan, 5e-324, 1.0, 1e308, 1e-308, 3.0]),
                  np.array([1.0, 1.0, 0.0, -0.0, 2.0, np.inf, 1.0, 1.0, 5e-324, 1e-10, 1e10, 3.0])))
    with np.errstate(all="ignore"):
        for x, y in pairs:
            ref = x / y
            out = hc.div_rn(x, y)
            same = (out.view(np.uint64) == ref.view(np.uint64)) | (np.isnan(out) & np.isnan(ref))
            assert same.all(), (x[~same][:3], y[~same][:3], out[~same][:3], ref[~same][:3])


def _stress_fixtures(per_noise=1):
    """The near-degenerate robustness sets (tests/golden/stress): the first instances of every noise
    level of both modes."""
    import json
    import os

    d = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "stress")
    seen, out = {}, []
    for e in json.load(open(os.path.join(d, "manifest.json"))):
        key = (e["mode"], e["noise"])
        if seen.get(key, 0) < per_noise:
            seen[key] = seen.get(key, 0) + 1
            out.append((e, json.load(open(os.path.join(d, e["file"])))))
    return out


def test_device_cut_logic_on_stress_sets(hc, oracle, fns):
    """Active tets of the robustness sets (four spheres, or spheres and a zero function, whose
    centres differ by 1e-7 to 1e-6, on a 99^3-cube grid): every variant of the device cut either
    defers or reproduces the oracle's record."""
    rng = np.random.default_rng(18)
    for e, specs in _stress_fixtures():
        funcs = fns.make_functions(specs)
        pts, tets = fns.generate_tet_mesh(e["resolution"])
        fv = oracle.sample(funcs, pts, threads=4)
        r = oracle.run(e["mode"], pts, tets, fv, threads=4)
        si, fit = r["start_index"], r["func_in_tet"]
        active = np.flatnonzero(np.diff(si) > 0)
        for t in rng.choice(active, size=min(120, len(active)), replace=False):
            rows = fv[tets[t]][:, fit[si[t]:si[t + 1]]].T.copy()
            ref = bytes(r["rec_bytes"][r["rec_offsets"][t]:r["rec_offsets"][t + 1]])
            _agree(hc, oracle, e["mode"], rows)
            got, _ = hc.cut(e["mode"], rows, True)
            assert got == ref, (e["file"], int(t))


def test_device_cut_logic_on_paper_examples(hc, oracle, fns):
    """The reference's paper examples (tests/golden/examples): inverse-CSG models of planes,
    cylinders and tori, and 18 spheres in both modes, on their 99^3-cube grids.  Up to 40 active
    tets of every active-function count, through every variant of the device cut."""
    import json
    import os

    d = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "examples")
    rng = np.random.default_rng(19)
    for e in json.load(open(os.path.join(d, "manifest.json"))):
        funcs = fns.make_functions(json.load(open(os.path.join(d, e["file"]))))
        pts, tets = fns.generate_tet_mesh(e["resolution"], *e["bbox"])
        fv = oracle.sample(funcs, pts, threads=4)
        r = oracle.run(e["mode"], pts, tets, fv, threads=4)
        si, fit = r["start_index"], r["func_in_tet"]
        k = np.diff(si)
        for kk in np.unique(k[k > 0]):
            pick = np.flatnonzero(k == kk)
            for t in rng.choice(pick, size=min(40, len(pick)), replace=False):
                rows = fv[tets[t]][:, fit[si[t]:si[t + 1]]].T.copy()
                ref = bytes(r["rec_bytes"][r["rec_offsets"][t]:r["rec_offsets"][t + 1]])
                _agree(hc, oracle, e["mode"], rows)
                got, _ = hc.cut(e["mode"], rows, True)
                assert got == ref, (e["file"], int(t))


def test_robust_test_classification(hc):
    """The robust test's per-tet outcome (robust.cuh, src/implicit_arrangement.cpp:137-243): exact cuts
    agree in both plane orders; a forged count mismatch is type 1, a forged failure of the cut in the
    given order type 2, of the reversed order type 3, in both modes."""
    rng = np.random.default_rng(77)
    for mode in ("ia", "mi"):
        for trial in range(40):
            k = int(rng.integers(2 if mode == "mi" else 1, 7))
            rows = rng.normal(size=(k, 4)) if trial % 2 else rng.integers(-2, 3, size=(k, 4)).astype(np.float64)
            assert hc.robust(mode, rows) == 0
            assert hc.robust(mode, rows, forge=1) == 1
            assert hc.robust(mode, rows, forge=2) == 2
            assert hc.robust(mode, rows, forge=3) == 3
