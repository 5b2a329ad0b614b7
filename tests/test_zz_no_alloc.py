"""The allocation-free batched solve (bm_dgbsv_batched_noalloc) against bm_dgbsv_batched.

Callers that cannot allocate device memory at solve time (real-time loops that must not
block on an allocator, hosts whose memory belongs to another runtime's pool) use the
allocation-free entry point: it takes only inputs and outputs and keeps its scratch
(work counter and longest-first order) in a static device array.  This checks, through
the C ABI, that two calls in a row give exactly what the regular entry point gives, so
the scratch left over from one call does not leak into the next.  This file is
collected last on purpose.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _make_batch(bm, gpu, rng, count):
    n = np.exp(rng.uniform(np.log(16), np.log(2000), count)).astype(np.int64)
    kl = rng.integers(0, 49, count)
    ku = rng.integers(0, 49, count)
    nrhs = rng.integers(1, 5, count)
    batch = bm.BandedBatch(n, kl, ku, nrhs, torch.float64, gpu)
    bands, rhs = [], []
    for s in range(count):
        d = rng.standard_normal((kl[s] + ku[s] + 1, n[s]))
        if s % 3:  # a third of the systems are not diagonally dominant: pivoting is exercised
            d[ku[s], :] += 2 * (kl[s] + ku[s])
        bands.append(torch.from_numpy(d).to(gpu))
        rhs.append(torch.from_numpy(rng.standard_normal((n[s], nrhs[s]))).to(gpu))
    return batch, bands, rhs


def _load(batch, bands, rhs):
    batch.AB.zero_()
    for s in range(batch.count):
        batch.matrix_band(s).copy_(bands[s])
        batch.rhs(s).copy_(rhs[s])
    batch.ipiv.fill_(-7)
    batch.info.fill_(-7)


def _same(a, b):
    """Bitwise-equal values; NaN in the same places counts as equal (unpivoted kl = 0
    systems can overflow in back substitution)."""
    return np.array_equal(a.cpu().numpy(), b.cpu().numpy(), equal_nan=True)


def _noalloc(bm, batch):
    L = bm._lib.load()
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    st = L.bm_dgbsv_batched_noalloc(batch.count, p(batch.descs), p(batch.AB), p(batch.ipiv), p(batch.B),
                                    p(batch.info), batch.max_kl, batch.max_ku,
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, L.bm_last_error()


def test_noalloc_matches_regular_entry_point_twice(bm, gpu):
    rng = np.random.default_rng(2024)
    batch, bands, rhs = _make_batch(bm, gpu, rng, 300)
    _load(batch, bands, rhs)
    batch.factor_solve()  # bm_dgbsv_batched, caller-provided counter and order
    torch.cuda.synchronize()
    ref_B, ref_ipiv, ref_info = batch.B.clone(), batch.ipiv.clone(), batch.info.clone()
    ref_AB = batch.AB.clone()
    for call in range(2):
        _load(batch, bands, rhs)
        _noalloc(bm, batch)
        torch.cuda.synchronize()
        assert torch.equal(batch.info, ref_info), call
        assert torch.equal(batch.ipiv, ref_ipiv), call
        assert _same(batch.AB, ref_AB), call
        assert _same(batch.B, ref_B), call


def test_noalloc_rejects_oversized_batches(bm, gpu):
    L = bm._lib.load()
    dummy = torch.zeros(16, dtype=torch.int64, device=gpu)
    p = ctypes.c_void_p(dummy.data_ptr())
    st = L.bm_dgbsv_batched_noalloc(65537, p, p, p, p, p, 1, 1, ctypes.c_void_p(0))
    assert st == bm._lib.BM_ERR_UNSUPPORTED
    assert b"65536" in L.bm_last_error()
