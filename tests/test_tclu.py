"""The tensor-core FP32 banded LU (bm_sgbtrf_tc) and the single-system refined solve
(bm_dsgbsv) against the oracle.

The FP32 factorization is blocked and its trailing updates are TF32 tensor-core
products with hi/lo-split operands, so it is not dgbtf2's operation order; it is
checked by what a factorization must deliver: the FP32 factors, used in the FP64
dgbtrs oracle, solve A x = b to a backward error of FP32 size (<= 5e-5 here, against
O(1) for a wrong factor), the pivots agree with dgbtf2's on at least 99% of the
columns (the pivot rule takes the largest |a| to 2^-15 relative), and a zero column
is reported in info exactly as dgbtf2 reports it.  The refined solve must reach the
requested backward error (1e-10) and agree with the FP64 solution to kappa * 1e-10.
"""
import ctypes

import numpy as np
import pytest
import torch


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def test_dsgbsv_argument_codes(bm):
    L = bm._lib.load()
    f = ctypes.c_void_p(256)  # never dereferenced: every call stops at an argument check
    s = ctypes.c_void_p(0)

    def ds(n=8, kl=4, ku=4, nrhs=1, ldab=9, ldb=8, ldx=8, tol=1e-10, maxit=5, work=f):
        return L.bm_dsgbsv(n, kl, ku, nrhs, f, ldab, f, ldb, f, ldx, f, f, work, ctypes.c_double(tol), maxit, f, f, f,
                           s)

    assert ds(n=-1) == -1
    assert ds(kl=-1) == -2
    assert ds(ku=-1) == -3
    assert ds(nrhs=-1) == -4
    assert ds(ldab=8) == -6
    assert ds(ldb=7) == -8
    assert ds(ldx=7) == -10
    assert ds(work=None) == -13
    assert ds(tol=-1.0) == -14
    assert ds(maxit=-1) == -15
    assert ds(kl=200, ku=100, ldab=301) == bm._lib.BM_ERR_UNSUPPORTED
    assert L.bm_sgbtrf_tc(8, 4, 4, f, 8, f, 17, f, f, s) == -5
    assert L.bm_sgbtrf_tc(8, 4, 4, f, 9, f, 12, f, f, s) == -7
    assert L.bm_sgbtrf_tc(8, 4, 4, f, 9, f, 17, f, f, s) == bm._lib.BM_ERR_UNSUPPORTED  # kl + ku < 64


def _band(rng, n, kl, ku, shift):
    d = rng.standard_normal((kl + ku + 1, n))
    d[ku] += shift
    return d


def _tc_factor(bm, gpu, data, n, kl, ku):
    L = bm._lib.load()
    A = torch.from_numpy(np.ascontiguousarray(data.T)).to(gpu)  # column-major (kl+ku+1) x n, lda = kl+ku+1
    ldf = 2 * kl + ku + 1
    F = torch.zeros(n, ldf, dtype=torch.float32, device=gpu)
    ipiv = torch.zeros(n, dtype=torch.int64, device=gpu)
    info = torch.full((1,), -5, dtype=torch.int64, device=gpu)
    st = L.bm_sgbtrf_tc(n, kl, ku, _p(A), kl + ku + 1, _p(F), ldf, _p(ipiv), _p(info),
                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, L.bm_last_error()
    torch.cuda.synchronize()
    return F.cpu().numpy().T.astype(np.float64), ipiv.cpu().numpy(), int(info.item())


def _berr(orc, data, n, kl, ku, x, b):
    r = orc.gbmv("N", n, n, kl, ku, 1.0, data, x) - b
    rows = orc.gbmv("N", n, n, kl, ku, 1.0, np.abs(data), np.ones(n))
    return float(np.abs(r).max() / (rows.max() * np.abs(x).max() + np.abs(b).max()))


@pytest.mark.gpu
@pytest.mark.parametrize("n,kl,ku,shift", [(4000, 128, 128, 16.0), (1000, 32, 32, 0.0), (777, 130, 120, 16.0),
                                           (300, 224, 32, 40.0), (64, 40, 30, 0.0), (33, 100, 156, 0.0),
                                           (5, 60, 4, 0.0), (2500, 64, 0, 0.0), (2000, 1, 200, 8.0),
                                           (1111, 96, 160, 0.0)])
def test_tc_factorization(bm, gpu, orc, n, kl, ku, shift):
    rng = np.random.default_rng(n + 7 * kl + ku)
    data = _band(rng, n, kl, ku, shift)
    F, ipiv, info = _tc_factor(bm, gpu, data, n, kl, ku)
    assert info == 0
    b = rng.standard_normal(n)
    x = orc.gbtrs("N", n, kl, ku, F, ipiv, b)
    assert _berr(orc, data, n, kl, ku, x, b) <= 5e-5
    _, ip64, _ = orc.gbtf2(n, n, kl, ku, orc.lu_storage(data, n, kl, ku))
    assert (ipiv == ip64).mean() >= 0.99, f"pivots agree on {(ipiv == ip64).mean():.4f}"


@pytest.mark.gpu
def test_tc_factorization_zero_column(bm, gpu, orc):
    n, kl, ku = 500, 70, 40
    rng = np.random.default_rng(3)
    data = _band(rng, n, kl, ku, 2.0 * (kl + ku))
    c = 237
    for r in range(kl + ku + 1):  # column c of A is zero
        data[r, c] = 0.0
    F, ipiv, info = _tc_factor(bm, gpu, data, n, kl, ku)
    _, _, info64 = orc.gbtf2(n, n, kl, ku, orc.lu_storage(data, n, kl, ku))
    assert info == info64 == c + 1


@pytest.mark.gpu
@pytest.mark.parametrize("n,kl,ku,nrhs", [(20000, 128, 128, 1), (3000, 130, 120, 3), (5000, 5, 7, 2),
                                          (700, 40, 60, 1)])
def test_dsgbsv_refines_to_tolerance(bm, gpu, orc, n, kl, ku, nrhs):
    """kappa ~ 1e4..1e6 (randn + 16 I for the wide bands): one or more corrections reach
    1e-10; the narrow band takes the FP32 dgbtf2-order factorization."""
    g = torch.Generator(device=gpu)
    g.manual_seed(n + kl)
    A = bm.BandedMatrix(bm.band_storage(kl + ku + 1, n, torch.float64, gpu), n, kl, ku)
    A.data.normal_(generator=g)
    A.data[ku] += 16.0 if kl + ku >= 64 else 4.0
    B = torch.randn(n, nrhs, dtype=torch.float64, device=gpu, generator=g)
    x, st = bm.solve_refined(A, B if nrhs > 1 else B[:, 0], tol=1e-10, maxit=20)
    torch.cuda.synchronize()
    assert int(st["info"]) == 0
    assert float(st["berr"]) <= 1e-10
    X = x.reshape(n, nrhs).cpu().numpy()
    data = A.data.cpu().numpy()
    Bh = B.cpu().numpy()
    LU, ip, _ = orc.gbtf2(n, n, kl, ku, orc.lu_storage(data, n, kl, ku))
    for c in range(nrhs):
        assert _berr(orc, data, n, kl, ku, X[:, c], Bh[:, c]) <= 1.5e-10
        x64 = orc.gbtrs("N", n, kl, ku, LU, ip, Bh[:, c])
        assert np.abs(X[:, c] - x64).max() <= 1e-4 * np.abs(x64).max()


@pytest.mark.gpu
def test_dsgbsv_singular_reports_info(bm, gpu):
    n, kl, ku = 400, 64, 64
    A = bm.BandedMatrix(bm.band_storage(kl + ku + 1, n, torch.float64, gpu), n, kl, ku)
    A.data.normal_()
    A.data[:, 99] = 0.0
    b = torch.randn(n, dtype=torch.float64, device=gpu)
    x, st = bm.solve_refined(A, b)
    assert int(st["info"]) == 100
    assert int(st["iters"]) == 0 and float(st["berr"]) == float("inf")


@pytest.mark.gpu
def test_dsgbsv_full_size_l128(bm, gpu):
    """n = 2^20, l = u = 128, randn + 16 I (kappa ~ 1e6): backward error <= 1e-10 checked
    on the host with SciPy's dgbmv, and the solution against SciPy's dgbtrf/dgbtrs."""
    from scipy.linalg import blas, lapack

    n, l = 1 << 20, 128
    g = torch.Generator(device=gpu)
    g.manual_seed(21)
    A = bm.BandedMatrix(bm.band_storage(2 * l + 1, n, torch.float64, gpu), n, l, l)
    A.data.normal_(generator=g)
    A.data[l] += 16.0
    b = torch.randn(n, dtype=torch.float64, device=gpu, generator=g)
    x, st = bm.solve_refined(A, b, tol=1e-10)
    torch.cuda.synchronize()
    assert int(st["info"]) == 0 and float(st["berr"]) <= 1e-10
    data = np.asfortranarray(A.data.cpu().numpy())
    xh, bh = x.cpu().numpy(), b.cpu().numpy()
    r = blas.dgbmv(n, n, l, l, 1.0, data, xh) - bh
    rows = blas.dgbmv(n, n, l, l, 1.0, np.abs(data), np.ones(n))
    assert np.abs(r).max() / (rows.max() * np.abs(xh).max() + np.abs(bh).max()) <= 1e-10
    AB = np.zeros((3 * l + 1, n), order="F")
    AB[l:] = data
    LU, ip, info = lapack.dgbtrf(AB, l, l, overwrite_ab=1)
    xo, _ = lapack.dgbtrs(LU, l, l, bh, ip)
    assert np.abs(xh - xo).max() <= 1e-6 * np.abs(xo).max()
