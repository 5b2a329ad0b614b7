"""Banded LU on the GPU (bm_{d,s}gbtrf / gbtrs / gbsv_batched) against the oracle.

The factorization reproduces dgbtf2 operation for operation, so factors and pivots
must equal the oracle's bit for bit; solves likewise ('T' with kl > 16 uses a tree
reduction and is checked to 1e-12).  Cases follow test/test_bandedlu.jl (5x5 (1,1)
L/U/p, transposed and multiple right-hand sides, non-square errors, zero sizes) plus
sweeps over n, kl, ku with and without diagonal dominance (pivoting exercised).
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
    if rows * n:
        d.copy_(torch.from_numpy(np.ascontiguousarray(data_np)))
    return bm.BandedMatrix(d, m, l, u)


def rel(a, b):
    b = np.asarray(b)
    s = np.abs(b).max() if b.size else 1.0
    return float(np.abs(np.asarray(a) - b).max() / (s if s > 0 else 1.0)) if b.size else 0.0


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n,l,u,shift", [(1, 0, 0, 0.0), (2, 1, 1, 0.0), (5, 1, 1, 0.0), (50, 2, 3, 0.0),
                                         (300, 4, 3, 0.0), (300, 4, 3, 10.0), (200, 30, 2, 0.0), (200, 2, 30, 0.0),
                                         (257, 33, 70, 0.0), (400, 64, 64, 0.0), (1000, 7, 0, 0.0),
                                         (1000, 0, 7, 0.0), (10000, 4, 3, 10.0), (3000, 16, 16, 0.0),
                                         # every register-window size class of kl and kl + ku
                                         (300, 40, 8, 0.0), (300, 49, 30, 0.0), (300, 20, 70, 0.0),
                                         (300, 12, 100, 0.0), (500, 56, 40, 5.0), (260, 6, 2, 0.0),
                                         (260, 12, 3, 0.0), (260, 24, 8, 0.0),
                                         # tiny bands (a lane per window element)
                                         (500, 1, 30, 0.0), (500, 3, 4, 0.0), (300, 2, 13, 0.0),
                                         (37, 4, 3, 0.0), (3, 2, 1, 0.0)])
def test_gbtrf_gbtrs_bitexact(bm, gpu, orc, dt, n, l, u, shift):
    rng = np.random.default_rng(n * 131 + l * 7 + u)
    data = rng.standard_normal((l + u + 1, n)).astype(dt)
    data[u, :] += dt(shift)
    A = dev_band(bm, data, n, l, u, gpu)
    F = bm.lu(A)
    LU, ipiv, info = orc.gbtf2(n, n, l, u, orc.lu_storage(data, n, l, u))
    assert F.info == info
    assert np.array_equal(F.ipiv.cpu().numpy(), ipiv), "pivots differ"
    got = F.factors.data.cpu().numpy()
    # compare every in-matrix position of the gbtrf storage (the top l rows hold fill-in)
    mask = orc.band_to_dense(np.ones_like(LU), n, l, l + u) != 0
    assert np.array_equal(orc.band_to_dense(got, n, l, l + u)[mask], orc.band_to_dense(LU, n, l, l + u)[mask])
    for nrhs in (1, 3):
        b = rng.standard_normal((n, nrhs)).astype(dt)
        bd = torch.from_numpy(b).to(gpu)
        xN = F.solve(bd).cpu().numpy()
        xT = F.T.solve(bd).cpu().numpy()
        refN = orc.gbtrs("N", n, l, u, LU, ipiv, b)
        refT = orc.gbtrs("T", n, l, u, LU, ipiv, b)
        assert np.array_equal(xN, refN, equal_nan=True)
        if l <= 16:
            assert np.array_equal(xT, refT, equal_nan=True)
        else:
            assert rel(xT, refT) < (1e-12 if dt == np.float64 else 1e-5)
    xv = F.solve(torch.from_numpy(b[:, 0].copy()).to(gpu)).cpu().numpy()
    assert np.array_equal(xv, refN[:, 0], equal_nan=True)


def test_lu_golden_through_gpu(bm, gpu, orc):
    """OpenBLAS dgbtrf/dgbtrs outputs (tests/golden) reproduced by the GPU factorization."""
    g = np.load(GOLD)
    t = 0
    while f"lu{t}_dims" in g:
        n, l, u, nrhs, info = (int(v) for v in g[f"lu{t}_dims"])
        A = dev_band(bm, g[f"lu{t}_data"], n, l, u, gpu)
        F = bm.lu(A)
        assert F.info == info
        assert np.array_equal(F.ipiv.cpu().numpy(), g[f"lu{t}_ipiv"]), t
        LU = g[f"lu{t}_LU"]
        got = F.factors.data.cpu().numpy()
        mask = orc.band_to_dense(np.ones_like(LU), n, l, l + u) != 0
        dg, dr = orc.band_to_dense(got, n, l, l + u)[mask], orc.band_to_dense(LU, n, l, l + u)[mask]
        if l >= 32 and u > 64:   # OpenBLAS uses blocked dgbtrf here; the GPU follows dgbtf2
            assert rel(dg, dr) < 1e-12
        else:
            assert np.array_equal(dg, dr), t
        bd = torch.from_numpy(g[f"lu{t}_b"]).to(gpu)
        assert rel(F.solve(bd).cpu().numpy(), g[f"lu{t}_xN"]) < 1e-12
        assert rel(F.T.solve(bd).cpu().numpy(), g[f"lu{t}_xT"]) < 1e-12
        t += 1


def test_cpu_runnable_case(bm, gpu, orc):
    """brandn(10000,10000,4,3) + 10I: x = A\\b against OpenBLAS at 1e-12, pivots bit-exact."""
    g = np.load(GOLD)
    data, b = g["cfg1_data"], g["cfg1_b"]
    n, l, u = 10000, 4, 3
    A = dev_band(bm, data, n, l, u, gpu)
    x = A.solve(torch.from_numpy(b).to(gpu)).cpu().numpy()
    assert rel(x, g["cfg1_x"]) < 1e-12
    F = bm.lu(A)
    assert np.array_equal(F.ipiv.cpu().numpy(), g["cfg1_ipiv"].astype(np.int64))
    Ad = orc.band_to_dense(data, n, l, u)
    assert orc.backward_error(Ad, x, b) < 1e-15


def test_reference_small_cases(bm, gpu, orc):
    """test/test_bandedlu.jl:26-53: L, U, p of a 5x5 (1,1) band against dense LU; solves."""
    import scipy.linalg

    rng = np.random.default_rng(0)
    data = rng.uniform(size=(3, 5))
    A = dev_band(bm, data, 5, 1, 1, gpu)
    Ad = orc.band_to_dense(data, 5, 1, 1)
    F = bm.lu(A)
    P, Lf, Uf = scipy.linalg.lu(Ad)
    assert np.allclose(F.L @ F.U, Ad[F.p - 1])
    assert np.allclose(F.U, Uf) and np.allclose(F.L, Lf)
    pf = np.argmax(P, axis=0) + 1
    assert np.array_equal(F.p, pf)
    assert F.issuccess()
    b = rng.uniform(size=5)
    bd = torch.from_numpy(b).to(gpu)
    assert np.allclose(F.solve(bd).cpu().numpy(), np.linalg.solve(Ad, b))
    assert np.allclose(F.T.solve(bd).cpu().numpy(), np.linalg.solve(Ad.T, b))
    assert np.allclose(F.adjoint().solve(bd).cpu().numpy(), np.linalg.solve(Ad.T, b))
    # b not overwritten by A \ b
    b0 = bd.clone()
    A.solve(bd)
    assert torch.equal(bd, b0)
    # multiple right-hand sides (a row-major (5,10) tensor: the call works on a copy)
    B = torch.from_numpy(rng.uniform(size=(5, 10))).to(gpu)
    assert np.allclose(F.solve(B).cpu().numpy(), np.linalg.solve(Ad, B.cpu().numpy()))
    assert np.allclose(bm.ldiv_(F, B.clone()).cpu().numpy(), np.linalg.solve(Ad, B.cpu().numpy()))


def test_non_square_and_sizes(bm, gpu, orc):
    rng = np.random.default_rng(1)
    for (m, n) in [(7, 5), (5, 7)]:
        data = rng.uniform(size=(3, n))
        A = dev_band(bm, data, m, 1, 1, gpu)
        F = bm.lu(A)
        LU, ipiv, info = orc.gbtf2(m, n, 1, 1, orc.lu_storage(data, n, 1, 1))
        assert np.array_equal(F.ipiv.cpu().numpy(), ipiv)
        b = torch.from_numpy(rng.uniform(size=m)).to(gpu)
        with pytest.raises(bm.DimensionMismatch):
            F.solve(b)
    F = bm.lu(dev_band(bm, rng.uniform(size=(3, 4)), 5, 1, 1, gpu))
    assert F.size() == (5, 4) and F.size(1) == 5 and F.size(2) == 4 and F.size(3) == 1
    with pytest.raises(IndexError):
        F.size(0)
    for (shape, bands) in [((0, 0), (1, 1)), ((0, 3), (1, 1)), ((0, 0), (-1, -2))]:
        A = bm.BandedMatrix.zeros(shape, bands, torch.float64, gpu)
        F = bm.lu(A)
        assert F.factors.shape == shape
        if shape[1] == 0:
            assert F.solve(torch.zeros(0, dtype=torch.float64, device=gpu)).numel() == 0


def test_singular_info(bm, gpu, orc):
    rng = np.random.default_rng(2)
    n, l, u = 60, 2, 2
    data = rng.standard_normal((l + u + 1, n))
    for r in range(l + u + 1):  # zero out column 20 of A entirely
        data[r, 20] = 0.0
    A = dev_band(bm, data, n, l, u, gpu)
    F = bm.lu(A)
    LU, ipiv, info = orc.gbtf2(n, n, l, u, orc.lu_storage(data, n, l, u))
    assert info > 0 and F.info == info and not F.issuccess()
    assert np.array_equal(F.ipiv.cpu().numpy(), ipiv)


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_batched_matches_single(bm, gpu, orc, dt):
    """Uneven batch (n log-uniform, kl/ku uniform in [0,40], 1-4 RHS): every system's
    factors, pivots and solution equal the single-system oracle's bit for bit."""
    rng = np.random.default_rng(3)
    count = 96
    n = np.exp(rng.uniform(np.log(8), np.log(600), count)).astype(np.int64)
    kl = rng.integers(0, 41, count)
    ku = rng.integers(0, 41, count)
    nrhs = rng.integers(1, 5, count)
    tdt = torch.float64 if dt == np.float64 else torch.float32
    batch = bm.BandedBatch(n, kl, ku, nrhs, tdt, gpu)
    datas, rhss = [], []
    for s in range(count):
        d = rng.standard_normal((kl[s] + ku[s] + 1, n[s])).astype(dt)
        d[ku[s], :] += dt(2 * (kl[s] + ku[s]))
        r = rng.standard_normal((n[s], nrhs[s])).astype(dt)
        batch.matrix_band(s).copy_(torch.from_numpy(d))
        batch.rhs(s).copy_(torch.from_numpy(r))
        datas.append(d)
        rhss.append(r)
    batch.factor_solve()
    torch.cuda.synchronize()
    info = batch.info.cpu().numpy()
    for s in range(count):
        LU, ipiv, inf = orc.gbtf2(n[s], n[s], kl[s], ku[s], orc.lu_storage(datas[s], n[s], kl[s], ku[s]))
        assert info[s] == inf
        assert np.array_equal(batch.pivots(s).cpu().numpy(), ipiv)
        x = orc.gbtrs("N", n[s], kl[s], ku[s], LU, ipiv, rhss[s])
        assert np.array_equal(batch.rhs(s).cpu().numpy(), x), s


def test_batched_graph_replay(bm, gpu):
    """The batched launch captures into a CUDA graph; replays re-solve refreshed inputs."""
    rng = np.random.default_rng(4)
    count = 64
    n = rng.integers(50, 300, count)
    kl = rng.integers(1, 20, count)
    ku = rng.integers(1, 20, count)
    nrhs = np.ones(count, dtype=np.int64)
    batch = bm.BandedBatch(n, kl, ku, nrhs, torch.float64, gpu)
    bands, rhs = [], []
    for s in range(count):
        d = rng.standard_normal((kl[s] + ku[s] + 1, n[s]))
        d[ku[s], :] += 2 * (kl[s] + ku[s])
        bands.append(torch.from_numpy(d).to(gpu))
        rhs.append(torch.from_numpy(rng.standard_normal((n[s], 1))).to(gpu))

    def load():
        batch.AB.zero_()
        for s in range(count):
            batch.matrix_band(s).copy_(bands[s])
            batch.rhs(s).copy_(rhs[s])

    load()
    batch.factor_solve()
    torch.cuda.synchronize()
    ref = batch.B.clone()
    load()
    g = batch.capture()
    for _ in range(2):
        load()
        g.replay()
        torch.cuda.synchronize()
        assert torch.equal(batch.B, ref)


def _uneven_batch(bm, gpu, seed, count, n_hi, band_hi, dt=torch.float64):
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(np.log(16), np.log(n_hi), count)).astype(np.int64)
    kl = rng.integers(0, band_hi + 1, count)
    ku = rng.integers(0, band_hi + 1, count)
    nrhs = rng.integers(1, 9, count)
    batch = bm.BandedBatch(n, kl, ku, nrhs, dt, gpu)
    g = torch.Generator(device=gpu)
    g.manual_seed(seed)
    for s in range(count):
        mb = batch.matrix_band(s)
        mb.normal_(generator=g)
        mb[int(ku[s])] += 2.0 * (kl[s] + ku[s]) + 1.0
        batch.rhs(s).normal_(generator=g)
    return batch


@pytest.mark.parametrize("tdt", [torch.float64, torch.float32])
def test_batched_schedules_bitexact(bm, gpu, tdt):
    """Two-part schedules (CTA width 4/8, any narrow/wide split) give the default
    launch's factors, pivots and solutions bit for bit: the group size only
    distributes the same operations."""
    batch = _uneven_batch(bm, gpu, 21, 120, 900, 70, tdt)
    AB0, B0 = batch.AB.clone(), batch.B.clone()
    batch.factor_solve()
    ref = (batch.AB.clone(), batch.ipiv.clone(), batch.B.clone(), batch.info.clone())
    ran = 0
    for warps in (4, 8):
        for cols in (0, 12, 33, 64, 1 << 30):
            batch.AB.copy_(AB0)
            batch.B.copy_(B0)
            batch.set_schedule(warps, cols)
            try:
                batch.factor_solve()
            except bm.BandedGPUError:  # this split's narrow slices do not fit in shared memory
                continue
            torch.cuda.synchronize()
            ran += 1
            got = (batch.AB, batch.ipiv, batch.B, batch.info)
            for a, b in zip(got, ref):
                assert torch.equal(a, b), (warps, cols)
    assert ran >= 6
    batch.set_schedule(None)


def test_batched_tune_picks_a_schedule_and_keeps_inputs(bm, gpu):
    """The autotuner times the candidates on the batch, restores its inputs and leaves
    the fastest schedule set; solving afterwards still gives the default results."""
    batch = _uneven_batch(bm, gpu, 22, 200, 1200, 48)
    AB0, B0 = batch.AB.clone(), batch.B.clone()
    batch.factor_solve()
    ref = batch.B.clone()
    batch.AB.copy_(AB0)
    batch.B.copy_(B0)
    best = batch.tune("plain")
    assert torch.equal(batch.AB, AB0) and torch.equal(batch.B, B0)
    assert best["warps"] in (4, 8) and len(best["candidates"]) >= 6
    assert best["ms"] == min(c["ms"] for c in best["candidates"])
    batch.factor_solve()
    assert torch.equal(batch.B, ref)
    again = batch.tune("plain")  # cached per batch shape
    assert again is best or again == best


def test_mixed_schedules_identical(bm, gpu):
    """The refined solve gives identical solutions, iterations and backward errors
    under every schedule."""
    batch = _uneven_batch(bm, gpu, 23, 96, 1500, 60)
    batch.solve_mixed(1e-10, 30)
    torch.cuda.synchronize()
    X0, it0, be0 = batch.X.clone(), batch.iters.clone(), batch.berr.clone()
    for warps in (4, 8):
        for cols in (0, 24, 1 << 30):
            batch.set_schedule(warps, cols)
            try:
                batch.solve_mixed(1e-10, 30)
            except bm.BandedGPUError:
                continue
            torch.cuda.synchronize()
            assert torch.equal(batch.X, X0) and torch.equal(batch.iters, it0) and torch.equal(batch.berr, be0), \
                (warps, cols)
    assert batch.berr.max().item() <= 1e-10


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("m,n,l,u,zero_cols", [(300, 300, 20, 20, (37, 38)), (260, 200, 25, 9, (16,)),
                                               (200, 260, 9, 25, (31, 100)), (500, 500, 40, 70, ()),
                                               (97, 97, 70, 3, (5, 50)), (129, 129, 18, 30, ())])
def test_cta_lu_panels_singular_and_rectangular(bm, gpu, orc, dt, m, n, l, u, zero_cols):
    """Bands wide enough for the CTA (panel) factorization: rectangular shapes, zero
    columns (exact zero pivots inside a panel) -- factors, pivots and info equal
    dgbtf2's bit for bit."""
    rng = np.random.default_rng(m + 3 * n + l)
    data = rng.standard_normal((l + u + 1, n)).astype(dt)
    for c in zero_cols:
        data[:, c] = 0.0
    A = dev_band(bm, data, m, l, u, gpu)
    F = bm.lu(A)
    LU, ipiv, info = orc.gbtf2(m, n, l, u, orc.lu_storage(data, n, l, u))
    assert F.info == info
    assert np.array_equal(F.ipiv.cpu().numpy(), ipiv)
    got = F.factors.data.cpu().numpy()
    mask = orc.band_to_dense(np.ones_like(LU), m, l, l + u) != 0
    assert np.array_equal(orc.band_to_dense(got, m, l, l + u)[mask], orc.band_to_dense(LU, m, l, l + u)[mask])


@pytest.mark.parametrize("dt,m,n,l,u,zero_cols", [(np.float64, 1500, 1500, 150, 150, ()),
                                                  (np.float64, 700, 600, 140, 160, (33, 300)),
                                                  (np.float32, 900, 900, 250, 240, (17,)),
                                                  (np.float64, 600, 700, 200, 100, ()),
                                                  (np.float64, 700, 700, 300, 60, (45,)),
                                                  (np.float64, 900, 900, 520, 30, (5, 600)),
                                                  (np.float32, 800, 800, 700, 20, ()),
                                                  (np.float32, 1000, 1000, 900, 10, ()),
                                                  (np.float64, 900, 900, 800, 10, (3,)),
                                                  (np.float64, 800, 800, 100, 300, ()),
                                                  (np.float64, 1000, 1000, 128, 128, (77,)),
                                                  (np.float64, 1200, 1100, 512, 40, ())])
def test_wide_band_panels_bitexact(bm, gpu, orc, dt, m, n, l, u, zero_cols):
    """Bands whose one-column window exceeds shared memory go through the panel +
    per-column replay launches (register panels of 1-4 rows per thread, and the
    shared-memory panel beyond): factors, pivots and info equal dgbtf2's bit for bit,
    and square systems solve ('N' bit-exact, 'T' to 1e-12 / 1e-5)."""
    rng = np.random.default_rng(m + n + l + u)
    data = rng.standard_normal((l + u + 1, n)).astype(dt)
    for c in zero_cols:
        data[:, c] = 0.0
    A = dev_band(bm, data, m, l, u, gpu)
    F = bm.lu(A)
    LU, ipiv, info = orc.gbtf2(m, n, l, u, orc.lu_storage(data, n, l, u))
    assert F.info == info
    assert np.array_equal(F.ipiv.cpu().numpy(), ipiv)
    got = F.factors.data.cpu().numpy()
    mask = orc.band_to_dense(np.ones_like(LU), m, l, l + u) != 0
    assert np.array_equal(orc.band_to_dense(got, m, l, l + u)[mask], orc.band_to_dense(LU, m, l, l + u)[mask])
    if m == n and info == 0:
        for nrhs in (1, 5):
            b = rng.standard_normal((n, nrhs)).astype(dt)
            bd = torch.from_numpy(b).to(gpu)
            assert np.array_equal(F.solve(bd).cpu().numpy(), orc.gbtrs("N", n, l, u, LU, ipiv, b))
            assert rel(F.T.solve(bd).cpu().numpy(), orc.gbtrs("T", n, l, u, LU, ipiv, b)) < \
                (1e-12 if dt == np.float64 else 1e-5)


def test_plan_matches_the_regular_batched_solve(bm, gpu):
    """bm_plan_create / bm_plan_execute_* (the library-owned autotuner) give, per system,
    exactly what the regular batched entry points give, for the plain and the refined
    solve; the plan's schedule is one of the timed candidates and is reused from the
    process cache for a batch of the same shape."""
    rng = np.random.default_rng(77)
    count = 200
    n = np.exp(rng.uniform(np.log(64), np.log(3000), count)).astype(np.int64)
    kl = rng.integers(1, 41, count)
    ku = rng.integers(1, 41, count)
    nrhs = rng.integers(1, 4, count)
    batch = bm.BandedBatch(n, kl, ku, nrhs, torch.float64, gpu)
    g = torch.Generator(device=gpu)
    g.manual_seed(3)
    for s in range(count):
        mb = batch.matrix_band(s)
        mb.normal_(generator=g)
        mb[int(ku[s])] += 2.0 * (kl[s] + ku[s])
        batch.rhs(s).normal_(generator=g)
    AB0, B0 = batch.AB.clone(), batch.B.clone()
    batch.factor_solve()
    torch.cuda.synchronize()
    ref_B, ref_ipiv = batch.B.clone(), batch.ipiv.clone()
    batch.AB.copy_(AB0)
    batch.B.copy_(B0)
    plan = batch.make_plan("plain")
    assert plan.candidates >= 2 and plan.tuned_ms > 0
    assert torch.equal(batch.AB, AB0) and torch.equal(batch.B, B0)  # timing ran on a copy
    plan.execute()
    torch.cuda.synchronize()
    assert torch.equal(batch.B, ref_B) and torch.equal(batch.ipiv, ref_ipiv)
    batch.AB.copy_(AB0)
    batch.B.copy_(B0)
    again = batch.make_plan("plain")  # same shape: the cached choice
    assert (again.schedule.n_wide, again.schedule.warps) == (plan.schedule.n_wide, plan.schedule.warps)
    again.close()
    plan.close()
    X_ref = batch.solve_mixed(1e-12, 20).clone()
    mp = batch.make_plan("mixed")
    batch.X.zero_()
    mp.execute(1e-12, 20)
    torch.cuda.synchronize()
    assert torch.equal(batch.X, X_ref)
    mp.close()


def _hard_quotients(rng, count):
    """(b, d) pairs whose quotient b/d lies within about eps * 2^-54 of an ulp from a
    rounding midpoint: for an odd 53-bit D and a small odd eps, M = eps / D mod 2^54 is
    odd and M*D = eps + B*2^54, so B/D = M/2^54 - eps/(D*2^54) with M/2^54 halfway
    between two doubles.  A quarter of the pairs instead has divisors with the largest
    significands, exponents beyond +-900 or subnormal numerators, where the solves take
    the plain division."""
    b = np.empty(count)
    d = np.empty(count)
    i = 0
    while i < count:
        D = int(rng.integers(2 ** 52, 2 ** 53)) | 1
        eps = int(rng.choice([-7, -5, -3, -1, 1, 3, 5, 7]))
        M = (eps * pow(D, -1, 2 ** 54)) % 2 ** 54
        B, rem = divmod(M * D - eps, 2 ** 54)
        if rem or not (2 ** 53 <= M < 2 ** 54 and 2 ** 52 <= B < 2 ** 53):
            continue
        e1, e2 = (int(x) for x in rng.integers(-200, 200, 2))
        b[i] = np.ldexp(float(B), e1) * (1 if rng.random() < 0.5 else -1)
        d[i] = np.ldexp(float(D), e2)
        i += 1
    k = count // 16
    d[:k] = np.ldexp(2.0 - np.arange(k) % 20 * 2.0 ** -52, rng.integers(-30, 30, k))  # top significands
    d[k:2 * k] *= 2.0 ** 700  # exponents beyond +-900
    b[2 * k:3 * k] = rng.standard_normal(k) * 2.0 ** -1030  # subnormal numerators
    b[3 * k:4 * k] = rng.standard_normal(k)
    d[3 * k:4 * k] = rng.standard_normal(k)
    return b, d


@pytest.mark.parametrize("ku", [0, 3, 50, 200])  # tiny, tiny, narrow, wide sweeps
def test_solve_division_is_correctly_rounded(bm, gpu, orc, ku):
    """The back substitution divides by U(j, j) through a staged reciprocal pair
    (Markstein's correction step) outside the ranges where it takes the plain division;
    on diagonal systems whose quotients sit next to rounding midpoints, 'N' and 'T'
    solves equal IEEE division bit for bit."""
    rng = np.random.default_rng(17 + ku)
    n = 4096
    b, d = _hard_quotients(rng, n)
    data = np.zeros((ku + 1, n))
    data[ku] = d
    A = dev_band(bm, data, n, 0, ku, gpu)
    F = bm.lu(A)
    assert F.info == 0
    want = b / d
    bd = torch.from_numpy(b.copy()).to(gpu)
    assert np.array_equal(F.solve(bd).cpu().numpy().view(np.int64), want.view(np.int64))
    assert np.array_equal(F.T.solve(bd).cpu().numpy().view(np.int64), want.view(np.int64))


@pytest.mark.parametrize("m,n,l,u", [(400, 400, 4, 3), (300, 260, 2, 1), (260, 300, 1, 30), (40, 33, 3, 4)])
def test_tiny_bands_special_values(bm, gpu, orc, m, n, l, u):
    """The tiny-band kernels (a lane per window element) on rectangular shapes, with zero
    columns (info), NaN and infinity in the band: factors, pivots and info equal
    dgbtf2's bit for bit (NaN where dgbtf2 has NaN), and square systems solve as dgbtrs."""
    rng = np.random.default_rng(m * 7 + n + l * 3 + u)
    data = rng.standard_normal((l + u + 1, n))
    data[:, n // 3] = 0.0
    data[u, n // 2] = np.nan
    data[max(u - 1, 0), 2 * n // 3] = np.inf
    data[u, 5] = 1e-310  # a subnormal pivot candidate
    A = dev_band(bm, data, m, l, u, gpu)
    F = bm.lu(A)
    LU, ipiv, info = orc.gbtf2(m, n, l, u, orc.lu_storage(data, n, l, u))
    assert F.info == info
    assert np.array_equal(F.ipiv.cpu().numpy(), ipiv)
    got = F.factors.data.cpu().numpy()
    mask = orc.band_to_dense(np.ones_like(LU), m, l, l + u) != 0
    assert np.array_equal(orc.band_to_dense(got, m, l, l + u)[mask], orc.band_to_dense(LU, m, l, l + u)[mask],
                          equal_nan=True)
    if m == n:
        b = rng.standard_normal((n, 2))
        x = F.solve(torch.from_numpy(b).to(gpu)).cpu().numpy()
        assert np.array_equal(x, orc.gbtrs("N", n, l, u, LU, ipiv, b), equal_nan=True)


@pytest.mark.parametrize("dt,m,n,l,u", [(np.float64, 700, 700, 130, 140), (np.float64, 600, 640, 300, 40),
                                        (np.float32, 520, 500, 260, 30)])
def test_wide_band_special_values_and_graph_capture(bm, gpu, orc, dt, m, n, l, u):
    """The wide-band panels (8 columns up to kl = 256, 4 above), launched with programmatic
    stream serialization: NaN, infinity and zero columns give dgbtf2's factors, pivots and
    info; the factorization captured in a CUDA graph and replayed gives the same bits."""
    rng = np.random.default_rng(m + 3 * n + l + u)
    data = rng.standard_normal((l + u + 1, n)).astype(dt)
    data[:, n // 4] = 0.0
    data[u, n // 2] = np.nan
    data[u - 1, 3 * n // 4] = np.inf
    A = dev_band(bm, data, m, l, u, gpu)
    F = bm.lu(A)
    LU, ipiv, info = orc.gbtf2(m, n, l, u, orc.lu_storage(data, n, l, u))
    assert F.info == info
    assert np.array_equal(F.ipiv.cpu().numpy(), ipiv)
    mask = orc.band_to_dense(np.ones_like(LU), m, l, l + u) != 0
    got = orc.band_to_dense(F.factors.data.cpu().numpy(), m, l, l + u)[mask]
    assert np.array_equal(got, orc.band_to_dense(LU, m, l, l + u)[mask], equal_nan=True)
    # the same factorization captured in a graph (a clean band, so that every step runs)
    data2 = rng.standard_normal((l + u + 1, n)).astype(dt)
    A2 = dev_band(bm, data2, m, l, u, gpu)
    F2 = bm.lu(A2)  # first call outside capture (per-device set-up)
    d = F2.factors.data
    src = torch.zeros_like(d)
    src[l:, :] = A2.data
    info2 = torch.zeros(1, dtype=torch.int64, device=gpu)
    s = torch.cuda.Stream(gpu)
    s.wait_stream(torch.cuda.current_stream(gpu))
    g = torch.cuda.CUDAGraph()
    prefix = "d" if dt == np.float64 else "s"
    with torch.cuda.graph(g, stream=s):
        d.copy_(src)
        bm._lib.call(f"bm_{prefix}gbtrf", m, n, l, u, d.data_ptr(), F2.factors.lda, F2.ipiv.data_ptr(),
                     info2.data_ptr(), s.cuda_stream)
    d.zero_()
    for _ in range(2):
        g.replay()
    torch.cuda.synchronize()
    LU2, ip2, inf2 = orc.gbtf2(m, n, l, u, orc.lu_storage(data2, n, l, u))
    assert int(info2.item()) == inf2
    assert np.array_equal(F2.ipiv.cpu().numpy(), ip2)
    got2 = orc.band_to_dense(d.cpu().numpy(), m, l, l + u)[mask]
    assert np.array_equal(got2, orc.band_to_dense(LU2, m, l, l + u)[mask])
