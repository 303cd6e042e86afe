"""ria_compute_arrangement_batch_noalloc against ria_compute_arrangement_batch (GPU).

The no-allocation entry point serves callers that cannot allocate device memory (their memory is
held by their own allocator, or cudaMalloc's possible device synchronization is not allowed in their
loop).  Its intermediate data lives in one fixed device array inside the library; this test gives it
device buffers for the inputs and outputs (allocated here by the test, not by the library) and
checks, on two calls in a row with different inputs, that its records equal those of the allocating
batch entry point byte for byte (the records are exact combinatorics, so the tolerance is equality).
The file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


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


def _run_noalloc(pkg, rows):
    import torch

    L = pkg.load()
    n = len(rows)
    offs = np.zeros(n + 1, dtype=np.int64)
    for i, r in enumerate(rows):
        offs[i + 1] = offs[i] + len(r)
    vals = np.concatenate(rows).reshape(-1)
    d_vals = torch.from_numpy(vals).cuda()
    d_off = torch.from_numpy(offs.astype(np.int32)).cuda()  # uint32 offsets (values < 2^31)
    cap = 6000 * n
    d_rec = torch.zeros(cap, dtype=torch.uint8, device="cuda")
    d_roff = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = L.ria_compute_arrangement_batch_noalloc(d_vals.data_ptr(), d_off.data_ptr(), n, d_rec.data_ptr(), cap,
                                                d_roff.data_ptr(), ctypes.c_void_p(stream))
    if st != 0:
        raise pkg.RiaError(st, L.ria_last_error().decode())
    roff = d_roff.cpu().numpy()
    rec = d_rec[: int(roff[-1])].cpu().numpy()
    return [bytes(rec[int(roff[i]):int(roff[i + 1])]) for i in range(n)]


def test_noalloc_equals_batch_on_two_calls(pkg):
    pkg.build()
    for seed, n in ((101, 3000), (202, 1700)):
        rows = _tets(seed, n)
        got = _run_noalloc(pkg, rows)
        ref = pkg.compute_arrangement_batch(rows)
        assert len(got) == len(ref)
        assert got == ref


def test_noalloc_rejects_too_many_tets(pkg):
    L = pkg.load()
    st = L.ria_compute_arrangement_batch_noalloc(1, 1, 4097, 1, 1, 1, None)
    assert st == pkg._lib.RIA_EINVAL
    assert b"4096" in L.ria_last_error()
