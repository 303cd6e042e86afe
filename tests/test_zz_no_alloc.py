"""ria_compute_arrangement_batch_noalloc on the GPU, against the oracle and the allocating entry point.

The no-allocation entry point serves callers that cannot allocate device memory (their memory is
held by their own allocator, or cudaMalloc's possible device synchronization is not allowed in their
loop).  Its intermediate data lives in one fixed device array inside the library; this test gives it
device buffers for the inputs and outputs (allocated here by the test, not by the library) and
checks:
  * on two calls in a row with different inputs, that its records equal the oracle's per-tet cut
    (oracle.ia_cut) and those of the allocating batch entry point byte for byte (the records are
    exact combinatorics, so the tolerance is equality);
  * that a caller buffer too small for the records gives RIA_ECAPACITY and leaves it untouched;
  * that records beyond the 8 MiB record space of the fixed array give RIA_ECAPACITY, and that the
    next call, which fits, is still exact (no state of the failed call leaks into it);
  * that malformed value offsets give RIA_EINVAL.
The file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SENTINEL = 0xAB


def _tets(seed, n):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        kind = i % 4
        k = int(rng.integers(1, 6))
        if kind == 0:
            rows = rng.normal(size=(k, 4))
        elif kind == 1:
            rows = rng.integers(-2, 3, size=(k, 4)).astype(np.float64)  # exact ties: exact variant
        elif kind == 2:
            p = rng.normal(size=4)
            rows = np.array([p, 2.0 * p, rng.normal(size=4)][: max(1, min(k, 3))])
        else:
            rows = rng.normal(size=(int(rng.integers(5, 8)), 4))  # large: capacity deferral
        out.append(np.ascontiguousarray(rows, dtype=np.float64))
    return out


def _offsets(rows):
    offs = np.zeros(len(rows) + 1, dtype=np.int64)
    for i, r in enumerate(rows):
        offs[i + 1] = offs[i] + len(r)
    return offs


def _call(pkg, vals, offs, n, cap):
    """One call through the C ABI on torch's current stream; returns (status, offsets, record buffer)."""
    import torch

    L = pkg.load()
    d_vals = torch.from_numpy(np.ascontiguousarray(vals, dtype=np.float64).reshape(-1)).cuda()
    d_off = torch.from_numpy(np.ascontiguousarray(offs).astype(np.int64).astype(np.uint32).view(np.int32)).cuda()
    d_rec = torch.full((max(cap, 1),), SENTINEL, dtype=torch.uint8, device="cuda")
    d_roff = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = L.ria_compute_arrangement_batch_noalloc(d_vals.data_ptr(), d_off.data_ptr(), n, d_rec.data_ptr(), cap,
                                                d_roff.data_ptr(), ctypes.c_void_p(stream))
    torch.cuda.synchronize()
    return st, d_roff.cpu().numpy(), d_rec.cpu().numpy()


def _run_noalloc(pkg, rows, cap=None):
    n = len(rows)
    cap = 6000 * n if cap is None else cap
    st, roff, rec = _call(pkg, np.concatenate(rows), _offsets(rows), n, cap)
    if st != 0:
        raise pkg.RiaError(st, pkg.load().ria_last_error().decode())
    return [bytes(rec[int(roff[i]):int(roff[i + 1])]) for i in range(n)]


def test_noalloc_equals_oracle_and_batch_on_two_calls(pkg, oracle):
    pkg.build()
    for seed, n in ((101, 3000), (202, 1700)):
        rows = _tets(seed, n)
        got = _run_noalloc(pkg, rows)
        assert len(got) == n
        assert got == [oracle.ia_cut(r) for r in rows]
        assert got == pkg.compute_arrangement_batch(rows)


def test_noalloc_small_caller_buffer(pkg, oracle):
    """A record buffer one byte short: RIA_ECAPACITY, and not one byte of the buffer is written."""
    rows = _tets(303, 600)
    need = sum(len(oracle.ia_cut(r)) for r in rows)
    st, roff, rec = _call(pkg, np.concatenate(rows), _offsets(rows), len(rows), need - 1)
    assert st == pkg._lib.RIA_ECAPACITY
    assert int(roff[-1]) == need  # the offsets still say how much room the call needs
    assert (rec == SENTINEL).all()
    assert _run_noalloc(pkg, rows, cap=need) == [oracle.ia_cut(r) for r in rows]


def test_noalloc_record_space_overflow_then_exact_call(pkg, oracle):
    """4096 tets of ten planes: about 15 MB of records, beyond the fixed 8 MiB record space."""
    rng = np.random.default_rng(404)
    rows = [rng.normal(size=(10, 4)) for _ in range(4096)]
    assert sum(len(oracle.ia_cut(r)) for r in rows) > (8 << 20)
    cap = 64 << 20
    st, _, rec = _call(pkg, np.concatenate(rows), _offsets(rows), len(rows), cap)
    assert st == pkg._lib.RIA_ECAPACITY
    assert b"8 MiB" in pkg.load().ria_last_error()
    assert (rec == SENTINEL).all()
    # the next call fits: its records must not depend on the failed one
    small = rows[:700]
    assert _run_noalloc(pkg, small) == [oracle.ia_cut(r) for r in small]
    rows2 = _tets(505, 2500)
    assert _run_noalloc(pkg, rows2) == [oracle.ia_cut(r) for r in rows2]


def test_noalloc_rejects_malformed_offsets(pkg):
    L = pkg.load()
    rows = _tets(606, 64)
    vals = np.concatenate(rows)
    offs = _offsets(rows)
    bad = offs.copy()
    bad[10], bad[11] = bad[11], bad[10]  # decreasing
    st, _, rec = _call(pkg, vals, bad, len(rows), 1 << 20)
    assert st == pkg._lib.RIA_EINVAL and b"value_offsets" in L.ria_last_error()
    assert (rec == SENTINEL).all()
    big = np.zeros(3, dtype=np.int64)
    big[1], big[2] = 61, 62  # 61 rows in one tet: beyond 60 active functions
    st, _, _ = _call(pkg, np.random.default_rng(1).normal(size=(62, 4)), big, 2, 1 << 20)
    assert st == pkg._lib.RIA_EINVAL


def test_noalloc_rejects_too_many_tets(pkg):
    L = pkg.load()
    st = L.ria_compute_arrangement_batch_noalloc(1, 1, 4097, 1, 1, 1, None)
    assert st == pkg._lib.RIA_EINVAL
    assert b"4096" in L.ria_last_error()
