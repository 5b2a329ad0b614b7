"""Format conversion on the GPU: sparse(A), bandwidths(S), BandedMatrix(S) and the
BandedRows copy, against host restatements of the reference's definitions.

sparse(A) must equal sparse(_banded_rowval(A), _banded_colval(A), _banded_nzval(A), m, n)
(ext/BandedMatricesSparseArraysExt.jl:7-9, src/banded/BandedMatrix.jl:796-836): the
triplets of every band slot, out-of-matrix rows clamped to the first / last row with
value 0, duplicates summed -- restated here with SciPy's COO -> CSC, which sums
duplicates and keeps explicit zeros.  Cases follow test/test_sparse.jl (sparse of a
BandedMatrix, bandwidths of sparse matrices including explicit zeros).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ref_sparse(data, m, n, l, u):
    import scipy.sparse as sp

    rows = l + u + 1
    kap, lam = np.meshgrid(np.arange(rows), np.arange(n), indexing="ij")
    ii = kap + lam - u  # 0-based row of slot (kappa, lambda)
    vals = np.where((ii >= 0) & (ii < m), data, 0.0)
    ii = np.clip(ii, 0, m - 1)
    S = sp.coo_matrix((vals.ravel(order="F"), (ii.ravel(order="F"), lam.ravel(order="F"))), shape=(m, n)).tocsc()
    S.sort_indices()
    return S


@pytest.mark.parametrize("m,n,l,u", [(50, 50, 2, 3), (40, 70, 5, 1), (70, 40, 0, 4), (30, 30, 0, 0),
                                     (10, 40, 2, 2), (1, 5, 3, 3)])
def test_sparse_matches_reference_structure(bm, gpu, m, n, l, u):
    rng = np.random.default_rng(m * n + l)
    data = rng.standard_normal((l + u + 1, n))
    data[0, 3] = -0.0
    A = bm.BandedMatrix(bm.band_storage(l + u + 1, n, torch.float64, gpu), m, l, u)
    A.data.copy_(torch.from_numpy(data))
    S = bm.sparse(A)
    R = _ref_sparse(data, m, n, l, u)
    assert np.array_equal(S.ccol_indices().cpu().numpy(), R.indptr)
    assert np.array_equal(S.row_indices().cpu().numpy(), R.indices)
    got, ref = S.values().cpu().numpy(), R.data
    assert np.array_equal(got, ref) and np.array_equal(np.signbit(got), np.signbit(ref))
    assert torch.equal(S.to_dense(), A.to_dense())


def test_sparse_bandwidths_and_back(bm, gpu):
    import scipy.sparse as sp

    rng = np.random.default_rng(3)
    for (m, n, l, u) in [(60, 60, 3, 7), (50, 80, 0, 12), (80, 50, 9, 0)]:
        D = np.zeros((m, n))
        for d in range(-l, u + 1):
            idx = np.arange(max(0, -d), min(m, n - d))
            D[idx, idx + d] = rng.standard_normal(len(idx))
        S = torch.from_numpy(D).to(gpu).to_sparse_csc()
        assert bm.sparse_bandwidths(S) == (l, u)
        A = bm.from_sparse(S)
        assert A.bandwidths() == (l, u)
        assert torch.equal(A.to_dense().cpu(), torch.from_numpy(D))
        with pytest.raises(ValueError):  # one band narrower than S's: its nonzeros there are dropped
            bm.from_sparse(S, (l - 1, u) if l > 0 else (l, u - 1))
    # explicit zeros do not count; an empty matrix has the bandwidths of Zeros
    Z = sp.csc_matrix((np.array([0.0, 0.0]), np.array([0, 5]), np.array([0, 1, 2] + [2] * 8)), shape=(10, 10))
    Sz = torch.sparse_csc_tensor(torch.from_numpy(Z.indptr.astype(np.int64)), torch.from_numpy(Z.indices.astype(np.int64)),
                                 torch.from_numpy(Z.data), (10, 10)).to(gpu)
    assert bm.sparse_bandwidths(Sz) == (-10, -10)
    E = torch.sparse_csc_tensor(torch.zeros(11, dtype=torch.int64), torch.zeros(0, dtype=torch.int64),
                                torch.zeros(0, dtype=torch.float64), (10, 10)).to(gpu)
    assert bm.sparse_bandwidths(E) == (-40320, -40320)


def test_banded_rows_copy(bm, gpu):
    rng = np.random.default_rng(5)
    m, n, l, u = 90, 100, 4, 6
    D = np.zeros((m, n))
    for d in range(-l, u + 1):
        idx = np.arange(max(0, -d), min(m, n - d))
        D[idx, idx + d] = rng.standard_normal(len(idx))
    R = np.zeros((m, l + u + 1))
    for i in range(m):
        for c in range(max(0, i - l), min(n, i + u + 1)):
            R[i, c - i + l] = D[i, c]
    A = bm.from_rows(torch.from_numpy(R).to(gpu), m, n, l, u)
    assert torch.equal(A.to_dense().cpu(), torch.from_numpy(D))
