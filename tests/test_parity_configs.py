"""Parity at the shapes of the benchmark workloads (GPU).

* Blocked regime: OpenBLAS switches to blocked dgbtrf (dgemm/dtrsm trailing updates)
  once kl reaches its block size, which is where the wide-band workloads live.  The GPU
  factorization (dgbtf2's operation order) is checked against OpenBLAS's pivots bit for
  bit and its factors and solutions to the tolerances of tests/test_oracle.py's
  BLOCKED_TOL, on tests/golden/blocked_golden.npz (l = u = 128 at n = 8192; the
  diffusion operator and an unshifted random band at l = u = 512, n = 4096), and
  against the dgbtf2 oracle bit for bit.
* Full size: the n = 2^20, l = u = 128 band (randn + 16 I) and the 512 x 512 diffusion
  operator (n = 262144, l = u = 512) are factored and solved on the GPU and by SciPy's
  OpenBLAS dgbtrf/dgbtrs on the host (the LAPACK routines lu!/ldiv! ccall,
  src/banded/BandedLU.jl:98, src/banded/linalg.jl:28): identical pivots, relative
  backward error <= 1e-12 for the GPU solution.
* The 4096-system uneven batch (n log-uniform in [256, 16384], l, u uniform in
  [1, 64], 1-8 right-hand sides, randn + 2(l+u) I), solved by one autotuned,
  graph-captured batched launch: 512 systems (a seeded 480 plus the 32 most expensive)
  equal the dgbtf2/dgbtrs oracle bit for bit (factors, pivots, solutions); the refined
  mixed-precision solve of the whole batch reaches backward error <= 1e-10 on every
  system, confirmed on the host for the sampled ones.
"""
import os
import sys

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
BLOCKED = os.path.join(HERE, "golden", "blocked_golden.npz")
BLOCKED_TOL = {"c4a": (1e-12, 1e-11), "c5": (1e-12, 1e-12), "r512": (1e-12, 1e-9)}


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def _inmatrix(n, kl, ku):
    """Mask of the gbtrf storage slots ((2kl+ku+1) x n) that hold entries of the matrix
    (row i = r - (kl+ku) + j inside 0..n-1); the corner slots outside it are never read."""
    r = np.arange(2 * kl + ku + 1)[:, None]
    i = r - (kl + ku) + np.arange(n)[None, :]
    return (i >= 0) & (i < n)


def _dev_band(bm, data, l, u, device):
    d = bm.band_storage(data.shape[0], data.shape[1], torch.float64, device)
    d.copy_(torch.from_numpy(np.ascontiguousarray(data)))
    return bm.BandedMatrix(d, data.shape[1], l, u)


def _berr_host(data, l, u, x, b):
    """||A x - b||_inf / (||A||_inf ||x||_inf + ||b||_inf) with SciPy's dgbmv (host)."""
    from scipy.linalg import blas

    n = data.shape[1]
    A = np.asfortranarray(data)
    r = blas.dgbmv(n, n, l, u, 1.0, A, x) - b
    rows = blas.dgbmv(n, n, l, u, 1.0, np.abs(A), np.ones(n))
    return float(np.abs(r).max() / (rows.max() * np.abs(x).max() + np.abs(b).max()))


@pytest.mark.parametrize("name", ["c4a", "c5", "r512"])
def test_blocked_regime_golden(bm, gpu, orc, name):
    import make_blocked_golden as mb

    gb = np.load(BLOCKED)
    data, l, u, b = mb.case_data(name, gb["c5_kfield"])
    n = data.shape[1]
    F = bm.lu(_dev_band(bm, data, l, u, gpu))
    x = F.solve(torch.from_numpy(b).to(gpu)).cpu().numpy()
    ipiv = F.ipiv.cpu().numpy()
    LU = F.factors.data.cpu().numpy()
    assert F.info == 0
    assert np.array_equal(ipiv, gb[f"{name}_pivoff"].astype(np.int64) + np.arange(1, n + 1)), "pivots differ"
    ftol, xtol = BLOCKED_TOL[name]
    assert _rel(LU[:, gb[f"{name}_cols"]], gb[f"{name}_LUcols"]) <= ftol
    assert _rel(x, gb[f"{name}_x"]) <= xtol
    assert _berr_host(data, l, u, x, b) <= 1e-12
    # and dgbtf2's operation order, bit for bit
    LUo, ipo, info = orc.gbtf2(n, n, l, u, orc.lu_storage(data, n, l, u))
    assert np.array_equal(ipiv, ipo)
    mask = _inmatrix(n, l, u)
    assert np.array_equal(LU[mask], LUo[mask])
    assert np.array_equal(x, orc.gbtrs("N", n, l, u, LUo, ipo, b))


def _full_size_check(bm, gpu, A, b):
    """GPU lu + solve of A against SciPy's dgbtrf/dgbtrs on the host."""
    from scipy.linalg import lapack

    n, l, u = A.n, A.l, A.u
    F = bm.lu(A)
    x = F.solve(b)
    torch.cuda.synchronize()
    assert F.info == 0
    ipiv = F.ipiv.cpu().numpy()
    xg = x.cpu().numpy()
    del F, x
    data = np.asfortranarray(A.data.cpu().numpy())
    bh = b.cpu().numpy()
    AB = np.zeros((2 * l + u + 1, n), order="F")
    AB[l:] = data
    LU, ip, info = lapack.dgbtrf(AB, l, u, overwrite_ab=1)
    assert info == 0
    assert np.array_equal(ipiv, ip.astype(np.int64) + 1), (
        f"{int((ipiv != ip + 1).sum())} pivots differ from OpenBLAS")
    xo, _ = lapack.dgbtrs(LU, l, u, bh, ip)
    del LU, AB
    be = _berr_host(data, l, u, xg, bh)
    assert be <= 1e-12, be
    return xg, xo


def test_config4a_full_size_plain_fp64(bm, gpu):
    """n = 2^20, l = u = 128, randn + 16 I, b randn: the plain FP64 path."""
    n, l = 1 << 20, 128
    g = torch.Generator(device=gpu)
    g.manual_seed(21)
    A = bm.BandedMatrix(bm.band_storage(2 * l + 1, n, torch.float64, gpu), n, l, l)
    A.data.normal_(generator=g)
    A.data[l] += 16.0
    b = torch.randn(n, dtype=torch.float64, device=gpu, generator=g)
    xg, xo = _full_size_check(bm, gpu, A, b)
    assert _rel(xg, xo) <= 1e-8  # kappa ~ 1e6


def test_config5_full_size_forward(bm, gpu):
    """The 512 x 512 diffusion operator (exp of a Gaussian field, correlation 16 cells),
    n = 262144, l = u = 512: the forward solve of the differentiated PDE workload."""
    G = 512
    kcell = np.exp(bm.pde.gaussian_field(G, 16.0, seed=11))
    A = bm.pde.diffusion_band(kcell, torch.float64, gpu)
    b = torch.from_numpy(np.random.default_rng(12).standard_normal(G * G)).to(gpu)
    xg, xo = _full_size_check(bm, gpu, A, b)
    assert _rel(xg, xo) <= 1e-10


def test_config3_batch_bitexact_and_refined(bm, gpu, orc):
    from bench import batched_config

    n, kl, ku, nrhs = batched_config()
    batch = bm.BandedBatch(n, kl, ku, nrhs, torch.float64, gpu)
    g = torch.Generator(device=gpu)
    g.manual_seed(5)
    for s in range(batch.count):
        mb = batch.matrix_band(s)
        mb.normal_(generator=g)
        mb[int(ku[s])] += 2.0 * (kl[s] + ku[s])
        batch.rhs(s).normal_(generator=g)
    AB0, B0 = batch.AB.clone(), batch.B.clone()
    cost = n * (2 * kl * (kl + ku) + kl) + nrhs * 2 * n * (2 * kl + ku + 1)
    top = np.argsort(-cost, kind="stable")[:32]
    rest = np.setdiff1d(np.arange(batch.count), top)
    sample = np.concatenate([top, np.random.default_rng(99).choice(rest, 480, replace=False)])
    inputs = {int(s): (batch.matrix_band(s).cpu().numpy(), batch.rhs(s).cpu().numpy()) for s in sample}

    batch.tune("plain")  # the autotuned schedule
    batch.AB.copy_(AB0)
    batch.B.copy_(B0)
    batch.factor_solve()  # device set-up outside capture
    graph = batch.capture()
    batch.AB.copy_(AB0)
    batch.B.copy_(B0)
    batch.info.fill_(-77)
    graph.replay()
    torch.cuda.synchronize()
    info = batch.info.cpu().numpy()
    assert (info == 0).all()
    for s in sample:
        s = int(s)
        data, b = inputs[s]
        N, L, U = int(n[s]), int(kl[s]), int(ku[s])
        LU, ip, inf = orc.gbtf2(N, N, L, U, orc.lu_storage(data, N, L, U))
        assert inf == 0
        assert np.array_equal(batch.pivots(s).cpu().numpy(), ip), s
        got = batch.band(s).data.cpu().numpy()
        mask = _inmatrix(N, L, U)
        assert np.array_equal(got[mask], LU[mask]), s
        x = orc.gbtrs("N", N, L, U, LU, ip, b)
        assert np.array_equal(batch.rhs(s).cpu().numpy(), x), s

    # the refined mixed-precision solve of the same batch (FP64 band and B untouched)
    batch.AB.copy_(AB0)
    batch.B.copy_(B0)
    batch.set_schedule(None)
    batch.solve_mixed(1e-10, 30)
    torch.cuda.synchronize()
    assert (batch.info.cpu().numpy() == 0).all()
    assert float(batch.berr.max()) <= 1e-10
    for s in sample[:64]:
        s = int(s)
        data, b = inputs[s]
        X = batch.solution(s).cpu().numpy()
        for c in range(b.shape[1]):
            assert _berr_host(data, int(kl[s]), int(ku[s]), X[:, c], b[:, c]) <= 1e-10, (s, c)
