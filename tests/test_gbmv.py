"""gbmv on the GPU (bm_dgbmv / bm_sgbmv through the C ABI) against the CPU oracle.

The kernel accumulates each output in the reference-BLAS order with fused
multiply-adds, so results must equal the oracle bit for bit (both precisions,
both transposes, every alpha/beta).  Shapes follow test/test_banded.jl:97-134
and the bandwidth sweep n = 2^24, l = u in {1, 8, 32}.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def dev_band(bm, data_np, m, l, u, device, lda=None):
    rows, n = data_np.shape
    d = bm.band_storage(rows, n, torch.float64 if data_np.dtype == np.float64 else torch.float32, device, lda=lda)
    d.copy_(torch.from_numpy(np.ascontiguousarray(data_np)))
    return bm.BandedMatrix(d, m, l, u)


def _np(dt):
    return np.float64 if dt == torch.float64 else np.float32


@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("m,n,kl,ku", [(50, 50, 2, 3), (40, 60, 3, 1), (60, 40, 0, 4), (1, 1, 0, 0), (7, 3, 5, 5),
                                       (1000, 1000, 1, 1), (3000, 2500, 17, 9), (4097, 4097, 32, 32),
                                       (20000, 20000, 8, 8), (5000, 5000, 0, 0), (300, 300, 100, 120)])
@pytest.mark.parametrize("alpha,beta", [(1.0, 0.0), (0.7, 1.3), (-2.0, 1.0), (1.5, -0.25)])
def test_gbmv_bitexact_vs_oracle(bm, gpu, orc, dt, trans, m, n, kl, ku, alpha, beta):
    rng = np.random.default_rng(m * 31 + n * 7 + kl * 3 + ku)
    nt = _np(dt)
    data = rng.uniform(-1, 1, (kl + ku + 1, n)).astype(nt)
    lx, ly = (n, m) if trans == "N" else (m, n)
    x = rng.standard_normal(lx).astype(nt)
    y0 = rng.standard_normal(ly).astype(nt)
    A = dev_band(bm, data, m, kl, ku, gpu)
    xd = torch.from_numpy(x).to(gpu)
    yd = torch.from_numpy(y0).to(gpu)
    bm.gbmv(trans, alpha, A, xd, beta, yd)
    ref = orc.gbmv(trans, m, n, kl, ku, alpha, data, x, beta, y0)
    got = yd.cpu().numpy()
    assert np.array_equal(got, ref), f"max diff {np.abs(got - ref).max()}"


def test_gbmv_golden_through_gpu(bm, gpu):
    g = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "lapack_golden.npz"))
    t = 0
    while f"gbmv{t}_dims" in g:
        m, n, kl, ku, tr = (int(v) for v in g[f"gbmv{t}_dims"])
        alpha, beta = (float(v) for v in g[f"gbmv{t}_ab"])
        A = dev_band(bm, g[f"gbmv{t}_data"], m, kl, ku, gpu)
        yd = torch.from_numpy(g[f"gbmv{t}_y0"].copy()).to(gpu)
        bm.gbmv("T" if tr else "N", alpha, A, torch.from_numpy(g[f"gbmv{t}_x"]).to(gpu), beta, yd)
        ref = g[f"gbmv{t}_y"]
        got = yd.cpu().numpy()
        assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max(), t
        if not tr:
            assert np.array_equal(got, ref), t
        t += 1


@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
def test_gbmv_strided_and_unaligned(bm, gpu, orc, dt):
    rng = np.random.default_rng(5)
    m, n, kl, ku = 777, 901, 6, 4
    nt = _np(dt)
    data = rng.standard_normal((kl + ku + 1, n)).astype(nt)
    A = dev_band(bm, data, m, kl, ku, gpu, lda=kl + ku + 3)  # lda > kl+ku+1
    x = rng.standard_normal(2 * n).astype(nt)
    y0 = rng.standard_normal(3 * m).astype(nt)
    xd = torch.from_numpy(x).to(gpu)
    yd = torch.from_numpy(y0).to(gpu)
    bm.gbmv("N", 0.5, A, xd[::2], 2.0, yd[::3])  # incx = 2, incy = 3
    ref = orc.gbmv("N", m, n, kl, ku, 0.5, data, x[::2].copy(), 2.0, y0[::3].copy())
    assert np.array_equal(yd.cpu().numpy()[::3], ref)
    # x one element off a 16-byte boundary: takes the generic kernel
    xd2 = torch.from_numpy(x).to(gpu)[1:n + 1]
    yd2 = torch.zeros(m, dtype=dt, device=gpu)
    bm.gbmv("N", 1.0, A, xd2, 0.0, yd2)
    ref2 = orc.gbmv("N", m, n, kl, ku, 1.0, data, x[1:n + 1].copy())
    assert np.array_equal(yd2.cpu().numpy(), ref2)


def test_gbmv_beta_zero_overwrites_nan(bm, gpu, orc):
    rng = np.random.default_rng(1)
    n, kl, ku = 1000, 3, 2
    data = rng.standard_normal((kl + ku + 1, n))
    A = dev_band(bm, data, n, kl, ku, gpu)
    x = torch.from_numpy(rng.standard_normal(n)).to(gpu)
    for trans in "NT":
        y = torch.full((n,), float("nan"), dtype=torch.float64, device=gpu)
        bm.gbmv(trans, 1.0, A, x, 0.0, y)
        assert torch.isfinite(y).all()


def test_mul_negative_bandwidths(bm, gpu, orc):
    """_banded_muladd! views (src/generic/matmul.jl:41-59); shapes of test/test_banded.jl:97-134."""
    rng = np.random.default_rng(2)
    for (l, u) in [(2, 3), (-2, 2), (2, -2), (2, -3), (-3, 2), (-1, 0)]:
        for (m, n) in [(10, 10), (10, 12), (12, 10)]:
            data = rng.standard_normal((max(0, l + u + 1), n))
            A = dev_band(bm, data, m, l, u, gpu)
            Ad = A.to_dense().cpu().numpy()
            x = rng.standard_normal(n)
            y = torch.from_numpy(rng.standard_normal(m)).to(gpu)
            y_ref = 0.3 * (Ad @ x) + 1.7 * y.cpu().numpy()
            bm.mul_(y, A, torch.from_numpy(x).to(gpu), 0.3, 1.7)
            assert np.allclose(y.cpu().numpy(), y_ref, rtol=1e-13, atol=1e-13), (l, u, m, n)
            xt = rng.standard_normal(m)
            yt = torch.zeros(n, dtype=torch.float64, device=gpu)
            bm.mul_t_(yt, A, torch.from_numpy(xt).to(gpu), 1.0, 0.0)
            assert np.allclose(yt.cpu().numpy(), Ad.T @ xt, rtol=1e-13, atol=1e-13), (l, u, m, n)
            if l + u + 1 > 0:
                assert np.allclose((A @ torch.from_numpy(x).to(gpu)).cpu().numpy(), Ad @ x, rtol=1e-13, atol=1e-13)


def test_gbmv_empty(bm, gpu):
    A = bm.BandedMatrix.zeros((0, 5), (1, 1), torch.float64, gpu)
    y = torch.zeros(0, dtype=torch.float64, device=gpu)
    bm.mul_(y, A, torch.ones(5, dtype=torch.float64, device=gpu))
    A = bm.BandedMatrix.zeros((5, 0), (1, 1), torch.float64, gpu)
    y = torch.ones(5, dtype=torch.float64, device=gpu)
    bm.mul_(y, A, torch.ones(0, dtype=torch.float64, device=gpu), 1.0, 2.0)
    assert torch.equal(y, torch.full((5,), 2.0, dtype=torch.float64, device=gpu))


def test_gbmv_illegal_arguments(bm, gpu):
    A = bm.BandedMatrix.zeros((5, 5), (1, 1), torch.float64, gpu)
    x = torch.ones(5, dtype=torch.float64, device=gpu)
    y = torch.ones(5, dtype=torch.float64, device=gpu)
    with pytest.raises(bm.BandedGPUError, match="argument 1"):
        bm.gbmv("X", 1.0, A, x, 0.0, y)
    with pytest.raises(bm.BandedGPUError, match="argument 8"):
        bm.gbmv("N", 1.0, A, x, 0.0, y, kl=3)  # lda = 3 < kl+ku+1


@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
@pytest.mark.parametrize("lu", [1, 8, 32])
def test_gbmv_full_size_windows(bm, gpu, orc, dt, lu):
    """n = 2^24, l = u in {1,8,32}: uniform(-1,1) band, randn x (the bandwidth sweep).  The whole
    product is checked bit for bit against the oracle on windows of rows (each window re-run
    on the CPU from the same band columns), plus y's checksum against a float64 reference."""
    n = 1 << 24
    g = torch.Generator(device=gpu)
    g.manual_seed(1234 + lu)
    A = bm.BandedMatrix(bm.band_storage(2 * lu + 1, n, dt, gpu), n, lu, lu)
    A.data.uniform_(-1.0, 1.0, generator=g)
    x = torch.randn(n, dtype=dt, device=gpu, generator=g)
    for trans in "NT":
        y = torch.empty(n, dtype=dt, device=gpu)
        bm.gbmv(trans, 1.0, A, x, 0.0, y)
        torch.cuda.synchronize()
        rng = np.random.default_rng(lu)
        starts = [0, n - 4096] + list(rng.integers(0, n - 4096, 6))
        for i0 in starts:
            i0 = int(i0)
            i1 = i0 + 4096
            if trans == "N":
                c0, c1 = max(0, i0 - lu), min(n, i1 + lu)
                blk = A.data[:, c0:c1].cpu().numpy()
                xs = x[c0:c1].cpu().numpy()
                # rows i0..i1 of A are a band of bandwidths (i0-c0, ...) over columns c0..c1
                ref = orc.gbmv("N", i1 - i0, c1 - c0, lu - (i0 - c0), lu + (i0 - c0), 1.0,
                               np.asfortranarray(blk), xs) if i0 - c0 <= lu else None
                got = y[i0:i1].cpu().numpy()
            else:
                r0, r1 = max(0, i0 - lu), min(n, i1 + lu)
                blk = A.data[:, i0:i1].cpu().numpy()
                xs = x[r0:r1].cpu().numpy()
                ref = orc.gbmv("T", r1 - r0, i1 - i0, lu + (i0 - r0), lu - (i0 - r0), 1.0,
                               np.asfortranarray(blk), xs)
                got = y[i0:i1].cpu().numpy()
            assert np.array_equal(got, ref), (trans, i0)
        del y
