"""Banded QR on the GPU (bm_{d,s}gbqrf, gbqr_lmul, tbsv) against the oracle.

The factorization follows _banded_qr! with reflector!/reflectorApply! operation for
operation, so factors and tau equal the oracle's bit for bit.  Cases follow
test/test_bandedqr.jl:7-69 (10x10 (3,2), 14x10, 10x14, 100x100 (3,4), 102x100,
100x102, tridiagonal) and the n = 2^18, l = u = 32 least-squares solve.
"""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "lapack_golden.npz")


def dev_band(bm, data_np, m, l, u, device):
    rows, n = data_np.shape
    dt = torch.float64 if data_np.dtype == np.float64 else torch.float32
    d = bm.band_storage(rows, n, dt, device)
    d.copy_(torch.from_numpy(np.ascontiguousarray(data_np)))
    return bm.BandedMatrix(d, m, l, u)


def oracle_qr(orc, data, m, n, l, u):
    D = np.zeros((2 * l + u + 1, n), dtype=data.dtype, order="F")
    D[l:, :] = data
    return orc.gbqrf(m, n, l, l + u, D)


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("m,n,l,u", [(10, 10, 3, 2), (14, 10, 3, 2), (10, 14, 3, 2), (100, 100, 3, 4),
                                     (102, 100, 3, 4), (100, 102, 3, 4), (100, 100, 1, 1), (5, 5, 0, 0),
                                     (1, 1, 0, 0), (2, 3, 1, 1), (300, 300, 32, 32), (2000, 2000, 8, 8),
                                     (500, 480, 20, 5)])
def test_gbqrf_bitexact(bm, gpu, orc, dt, m, n, l, u):
    rng = np.random.default_rng(m * 7 + n + l * 3 + u)
    data = rng.uniform(0, 1, (l + u + 1, n)).astype(dt)
    F = bm.qr(dev_band(bm, data, m, l, u, gpu))
    Fo, tau = oracle_qr(orc, data, m, n, l, u)
    got = F.factors.data.cpu().numpy()
    mask = orc.band_to_dense(np.ones_like(Fo), m, l, l + u) != 0
    dg, dr = orc.band_to_dense(got, m, l, l + u), orc.band_to_dense(Fo, m, l, l + u)
    assert np.array_equal(dg[mask], dr[mask])
    assert np.array_equal(F.tau.cpu().numpy(), tau)


def test_qr_golden_dgeqrf(bm, gpu, orc):
    """qr(A).factors and .tau against dense LAPACK dgeqrf (test/test_bandedqr.jl:34-36)."""
    g = np.load(GOLD)
    for t in range(6):
        m, n, l, u = (int(v) for v in g[f"qr{t}_dims"])
        F = bm.qr(dev_band(bm, g[f"qr{t}_data"], m, l, u, gpu))
        dense = orc.band_to_dense(F.factors.data.cpu().numpy(), m, l, l + u)
        mask = orc.band_to_dense(np.ones((2 * l + u + 1, n)), m, l, l + u) != 0
        qr = g[f"qr{t}_qr"]
        assert np.abs(dense[mask] - qr[mask]).max() <= 1e-12 * np.abs(qr).max(), t
        assert np.abs(F.tau.cpu().numpy() - g[f"qr{t}_tau"]).max() <= 1e-12, t
        if f"qr{t}_x" in g:
            x = F.solve(torch.from_numpy(g[f"qr{t}_b"]).to(gpu)).cpu().numpy()
            assert np.abs(x - g[f"qr{t}_x"]).max() <= 1e-10 * np.abs(g[f"qr{t}_x"]).max(), t


def test_qr_products_and_solve(bm, gpu, orc):
    """Q*(Q'*b) == b, Q'A[:,j] == R[:,j], qr(A)\\b == dense solve (square, tall, 2 RHS)."""
    rng = np.random.default_rng(5)
    for (m, n, l, u) in [(10, 10, 3, 2), (14, 10, 3, 2), (100, 100, 3, 4), (102, 100, 3, 4)]:
        data = rng.uniform(0, 1, (l + u + 1, n))
        A = dev_band(bm, data, m, l, u, gpu)
        Ad = orc.band_to_dense(data, m, l, u)
        F = bm.qr(A)
        b = torch.from_numpy(rng.uniform(size=m)).to(gpu)
        qtb = F.Q.adjoint() @ b
        assert torch.allclose(F.Q @ qtb, b, rtol=1e-13, atol=1e-13)
        R = F.R.cpu().numpy()
        QtA = (F.Q.T @ torch.from_numpy(Ad).to(gpu)).cpu().numpy()
        assert np.allclose(QtA[: min(m, n)], R, atol=1e-12)
        x = F.solve(b).cpu().numpy()
        assert np.allclose(x, np.linalg.lstsq(Ad, b.cpu().numpy(), rcond=None)[0], rtol=1e-10, atol=1e-12)
        B2 = torch.from_numpy(rng.uniform(size=(m, 2))).to(gpu)
        X2 = F.solve(B2).cpu().numpy()
        assert np.allclose(X2, np.linalg.lstsq(Ad, B2.cpu().numpy(), rcond=None)[0], rtol=1e-10, atol=1e-12)
        with pytest.raises(bm.DimensionMismatch):
            F.solve(torch.zeros(3, dtype=torch.float64, device=gpu))


def test_qr_tridiagonal_and_ldiv_dispatch(bm, gpu, orc):
    """qr of a tridiagonal band (test/test_bandedqr.jl:60-68) and A \\ b for a tall A (-> qr)."""
    rng = np.random.default_rng(6)
    n = 100
    data = rng.standard_normal((3, n))
    A = dev_band(bm, data, n, 1, 1, gpu)
    F = bm.qr(A)
    Fo, tau = oracle_qr(orc, data, n, n, 1, 1)
    assert np.array_equal(F.tau.cpu().numpy(), tau)
    m = 120
    data = rng.standard_normal((5, n))
    A = dev_band(bm, data, m, 2, 2, gpu)  # tall 120 x 100
    b = rng.standard_normal(m)
    x = A.solve(torch.from_numpy(b).to(gpu)).cpu().numpy()
    assert np.allclose(x, np.linalg.lstsq(orc.band_to_dense(data, m, 2, 2), b, rcond=None)[0], rtol=1e-10, atol=1e-12)


def test_qr_least_squares_full_size(bm, gpu, orc):
    """n = 2^18, l = u = 32 (the QR least-squares workload): factors bit-exact against the
    oracle, and the FP64 residual of x = qr(A) \\ b at the level of the backward error."""
    n, l, u = 1 << 18, 32, 32
    g = torch.Generator(device=gpu)
    g.manual_seed(7)
    A = bm.BandedMatrix(bm.band_storage(l + u + 1, n, torch.float64, gpu), n, l, u)
    A.data.normal_(generator=g)
    b = torch.randn(n, dtype=torch.float64, device=gpu, generator=g)
    F = bm.qr(A)
    x = F.solve(b)
    r = b.clone()
    bm.mul_(r, A, x, -1.0, 1.0)  # r = b - A x (FP64 gbmv)
    absA = bm.BandedMatrix(A.data.abs(), n, l, u)
    anorm = (absA @ torch.ones(n, dtype=torch.float64, device=gpu)).max().item()
    berr = r.abs().max().item() / (anorm * x.abs().max().item() + b.abs().max().item())
    assert berr < 1e-12, berr
    data = A.data.cpu().numpy()
    Fo, tau = oracle_qr(orc, data, n, n, l, u)
    assert np.array_equal(F.tau.cpu().numpy(), tau)
    got = F.factors.data.cpu().numpy()
    assert np.array_equal(got[:, 64:-64], Fo[:, 64:-64])


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_qr_lmul_bitexact(bm, gpu, orc, dt):
    """Q'b and Qb equal the oracle's banded_qr_lmul! restatement bit for bit (the
    reflector dot products in the factorization's four-way interleaved order)."""
    rng = np.random.default_rng(41)
    for (m, n, l, u, nrhs) in [(300, 300, 7, 5, 1), (520, 500, 20, 11, 3), (64, 64, 40, 2, 9)]:
        data = rng.standard_normal((l + u + 1, n)).astype(dt)
        F = bm.qr(dev_band(bm, data, m, l, u, gpu))
        Fo, tau = oracle_qr(orc, data, m, n, l, u)
        B = rng.standard_normal((m, nrhs)).astype(dt)
        for trans in ("T", "N"):
            ref = orc.gbqr_lmul(trans, m, n, l, l + u, Fo, tau, B.copy())
            Bd = torch.from_numpy(B.copy()).to(gpu)
            Q = F.Q.adjoint() if trans == "T" else F.Q
            got = (Q @ Bd).cpu().numpy()
            assert np.array_equal(got, ref), (m, n, l, u, trans)
