"""Mixed-precision refined batched solve (bm_dsgbsv_batched): FP32 factorization, FP64
residual and update.  Every system must reach the requested backward error, and the
solutions must agree with the FP64 oracle's to the accuracy the conditioning allows."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _fill(bm, gpu, rng, n, kl, ku, nrhs, shift_fn):
    batch = bm.BandedBatch(n, kl, ku, nrhs, torch.float64, gpu)
    data, rhs = [], []
    for s in range(batch.count):
        d = rng.standard_normal((kl[s] + ku[s] + 1, n[s]))
        d[ku[s], :] += shift_fn(s, d)
        r = rng.standard_normal((n[s], nrhs[s]))
        batch.matrix_band(s).copy_(torch.from_numpy(d))
        batch.rhs(s).copy_(torch.from_numpy(r))
        data.append(d)
        rhs.append(r)
    return batch, data, rhs


def _berr(orc, d, n, kl, ku, x, b):
    r = b - orc.gbmv("N", n, n, kl, ku, 1.0, d, x)
    A = np.abs(d)
    anorm = orc.gbmv("N", n, n, kl, ku, 1.0, A, np.ones(n)).max()
    return np.abs(r).max() / (anorm * np.abs(x).max() + np.abs(b).max())


def test_mixed_batched_reaches_tolerance(bm, gpu, orc):
    """Uneven, diagonally dominant systems (shift 2(kl+ku)), 1-4 right-hand sides."""
    rng = np.random.default_rng(11)
    count = 160
    n = np.exp(rng.uniform(np.log(32), np.log(3000), count)).astype(np.int64)
    kl = rng.integers(1, 65, count)
    ku = rng.integers(1, 65, count)
    nrhs = rng.integers(1, 5, count)
    batch, data, rhs = _fill(bm, gpu, rng, n, kl, ku, nrhs, lambda s, d: 2.0 * (kl[s] + ku[s]))
    batch.solve_mixed(tol=1e-10, maxit=30)
    torch.cuda.synchronize()
    assert int(batch.info.abs().max()) == 0
    berr = batch.berr.cpu().numpy()
    assert berr.max() <= 1e-10, berr.max()
    for s in range(0, count, 7):
        x = batch.solution(s).cpu().numpy()
        LU, ipiv, _ = orc.gbtf2(n[s], n[s], kl[s], ku[s], orc.lu_storage(data[s], n[s], kl[s], ku[s]))
        xr = orc.gbtrs("N", n[s], kl[s], ku[s], LU, ipiv, rhs[s])
        assert np.abs(x - xr).max() <= 1e-10 * np.abs(xr).max()
        for c in range(nrhs[s]):
            assert _berr(orc, data[s], n[s], kl[s], ku[s], x[:, c], rhs[s][:, c]) <= 1.01e-10
    # inputs untouched
    for s in range(0, count, 13):
        assert np.array_equal(batch.matrix_band(s).cpu().numpy(), data[s])
        assert np.array_equal(batch.rhs(s).cpu().numpy(), rhs[s])


def test_mixed_ill_conditioned_and_pivoting(bm, gpu, orc):
    """Non-dominant systems (pivoting) and shifts spreading kappa over 1e2..1e7: every
    system with kappa_inf < 1e6 must reach 1e-10."""
    rng = np.random.default_rng(12)
    count = 48
    n = np.full(count, 400)
    kl = rng.integers(2, 12, count)
    ku = rng.integers(2, 12, count)
    nrhs = np.ones(count, dtype=np.int64)
    shifts = [0.0, 0.5, 1.0, 2.0, 3.0, 5.0]
    batch, data, rhs = _fill(bm, gpu, rng, n, kl, ku, nrhs,
                             lambda s, d: shifts[s % len(shifts)] * np.sqrt(kl[s] + ku[s] + 1))
    batch.solve_mixed(tol=1e-10, maxit=60)
    torch.cuda.synchronize()
    berr = batch.berr.cpu().numpy()
    its = batch.iters.cpu().numpy()
    conds = np.array([np.linalg.cond(orc.band_to_dense(data[s], n[s], kl[s], ku[s]), np.inf)
                      for s in range(count)])
    ok = conds < 1e6
    assert ok.sum() >= 8 and (conds > 1e4).any()
    assert berr[ok].max() <= 1e-10, (berr[ok].max(), its[ok].max())
    for s in np.nonzero(ok)[0]:
        x = batch.solution(s).cpu().numpy()[:, 0]
        assert _berr(orc, data[s], n[s], kl[s], ku[s], x, rhs[s][:, 0]) <= 1.01e-10


def test_mixed_matches_fp64_systems_and_iterations(bm, gpu, orc):
    """FP32 factors with FP64 refinement reach the FP64 solution; iterations stay small
    for well-conditioned systems."""
    rng = np.random.default_rng(13)
    count = 32
    n = rng.integers(200, 1500, count)
    kl = rng.integers(1, 33, count)
    ku = rng.integers(1, 33, count)
    nrhs = rng.integers(1, 9, count)
    batch, data, rhs = _fill(bm, gpu, rng, n, kl, ku, nrhs, lambda s, d: 2.0 * (kl[s] + ku[s]))
    batch.solve_mixed(tol=1e-12, maxit=20)
    torch.cuda.synchronize()
    assert batch.berr.max().item() <= 1e-12
    assert batch.iters.max().item() <= 6


def test_single_system_refined_wide_and_conditioned(bm, gpu, orc):
    """solve_refined (Float32 LU, Float64 residuals) on a band whose Float64 window is
    too wide for one CTA and a shift giving kappa ~ 1e5..1e6: the backward error
    reaches 1e-10, and the solution matches the Float64 LU solve to kappa * 1e-10."""
    n, kl, ku = 4000, 130, 120
    g = torch.Generator(device=gpu)
    g.manual_seed(31)
    A = bm.BandedMatrix(bm.band_storage(kl + ku + 1, n, torch.float64, gpu), n, kl, ku)
    A.data.normal_(generator=g)
    A.data[ku] += 16.0
    b = torch.randn(n, dtype=torch.float64, device=gpu, generator=g)
    x, st = bm.solve_refined(A, b, tol=1e-10)
    assert int(st["info"]) == 0 and float(st["berr"]) <= 1e-10 and int(st["iters"]) >= 1
    F = bm.lu(A)
    x64 = F.solve(b)
    kappa = float(A.data.abs().sum(0).max()) * F.inv_norm1_estimate()
    assert 1e3 < kappa < 1e8, kappa
    assert float((x - x64).abs().max()) <= 10 * kappa * 1e-10 * float(x64.abs().max())
    r = b.clone()
    bm.mul_(r, A, x, -1.0, 1.0)
    anorm = float(A.data.abs().sum(0).max())
    assert float(r.abs().max()) / (anorm * float(x.abs().max()) + float(b.abs().max())) <= 1.5e-10


def test_mixed_small_zero_bandwidth_and_singular(bm, gpu, orc):
    """Systems shorter than one 16-column panel, zero bandwidths, bands at the blocked
    path's limits, and one singular system (a zero column): info reports the zero pivot
    and that system is not refined; every other system converges to the oracle's
    solution."""
    rng = np.random.default_rng(14)
    shapes = [(1, 0, 0), (2, 1, 0), (2, 0, 1), (5, 3, 3), (15, 2, 7), (16, 16, 0), (17, 0, 16), (33, 5, 1),
              (40, 12, 30), (100, 0, 0), (300, 63, 64), (257, 64, 31), (50, 4, 4)]
    n = np.array([s[0] for s in shapes])
    kl = np.array([s[1] for s in shapes])
    ku = np.array([s[2] for s in shapes])
    nrhs = rng.integers(1, 7, len(shapes))
    sing = len(shapes) - 1

    def shift(s, d):
        if s == sing:
            d[:, 3] = 0.0  # column 3 of A is zero: the factorization meets a zero pivot
            return 0.0
        return 2.0 * (kl[s] + ku[s]) + 1.0

    batch, data, rhs = _fill(bm, gpu, rng, n, kl, ku, nrhs, shift)
    batch.solve_mixed(tol=1e-10, maxit=30)
    torch.cuda.synchronize()
    info = batch.info.cpu().numpy()
    assert info[sing] == 4, info
    ok = np.arange(len(shapes)) != sing
    assert np.abs(info[ok]).max() == 0
    berr = batch.berr.cpu().numpy()
    assert berr[ok].max() <= 1e-10, berr
    assert batch.iters.cpu().numpy()[sing] == 0
    for s in np.nonzero(ok)[0]:
        x = batch.solution(s).cpu().numpy()
        LU, ipiv, _ = orc.gbtf2(n[s], n[s], kl[s], ku[s], orc.lu_storage(data[s], n[s], kl[s], ku[s]))
        xr = orc.gbtrs("N", n[s], kl[s], ku[s], LU, ipiv, rhs[s])
        assert np.abs(x - xr).max() <= 1e-10 * max(1.0, np.abs(xr).max()), s
