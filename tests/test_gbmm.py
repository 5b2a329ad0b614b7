"""Banded x banded products on the GPU (bm_dgbmm / bm_sgbmm) against the oracle.

Every C entry is accumulated like the column dgbmv of _gbmm! (src/banded/gbmm.jl:296-340),
so in-matrix entries equal the oracle's _gbmm! restatement bit for bit.  Cases follow
test/test_linalg.jl:138-325 (the {1,5,50} x {0,1,2,30} sweep, negative bands, NaN
overwrite, "not enough bands") and the n = 2^20, l = u = 16 product.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def dev_band(bm, data_np, m, l, u, device):
    rows, n = data_np.shape
    dt = torch.float64 if data_np.dtype == np.float64 else torch.float32
    d = bm.band_storage(rows, n, dt, device)
    if rows * n:
        d.copy_(torch.from_numpy(np.ascontiguousarray(data_np)))
    return bm.BandedMatrix(d, m, l, u)


def in_matrix(orc, data, m, l, u):
    return orc.band_to_dense(np.asarray(data), m, l, u)


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_gbmm_reference_sweep_bitexact(bm, gpu, orc, dt):
    """All n,nu,m in {1,5,50} and Al,Au,Bl,Bu in {0,1,2,30}, alpha=0.123, beta=0.456."""
    rng = np.random.default_rng(17)
    bad = []
    for n in (1, 5, 50):
        for nu in (1, 5, 50):
            for m in (1, 5, 50):
                for Al in (0, 1, 2, 30):
                    for Au in (0, 1, 2, 30):
                        for Bl in (0, 1, 2, 30):
                            for Bu in (0, 1, 2, 30):
                                A = rng.uniform(size=(Al + Au + 1, nu)).astype(dt)
                                B = rng.uniform(size=(Bl + Bu + 1, m)).astype(dt)
                                C = rng.uniform(size=(Al + Bl + Au + Bu + 1, m)).astype(dt)
                                ref = orc.gbmm_percol(n, nu, m, Al, Au, Bl, Bu, 0.123, A, B, 0.456, C)
                                Ad = dev_band(bm, A, n, Al, Au, gpu)
                                Bd = dev_band(bm, B, nu, Bl, Bu, gpu)
                                Cd = dev_band(bm, C, n, Al + Bl, Au + Bu, gpu)
                                bm.banded_mul_(Cd, Ad, Bd, 0.123, 0.456)
                                got = Cd.data.cpu().numpy()
                                l, u = Al + Bl, Au + Bu
                                if not np.array_equal(in_matrix(orc, got, n, l, u), in_matrix(orc, ref, n, l, u)):
                                    bad.append((n, nu, m, Al, Au, Bl, Bu))
    assert not bad, f"{len(bad)} cases differ, first {bad[:5]}"


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("alpha,beta", [(1.0, 0.0), (0.5, 2.0), (-1.25, 1.0)])
def test_gbmm_wide_c_and_scaling(bm, gpu, orc, dt, alpha, beta):
    """C with more bands than the product: extra bands are beta-scaled (gbmm.jl:286-288)."""
    rng = np.random.default_rng(3)
    n = nu = m = 300
    Al, Au, Bl, Bu = 3, 2, 4, 1
    Cl, Cu = Al + Bl + 3, Au + Bu + 2
    A = rng.standard_normal((Al + Au + 1, nu)).astype(dt)
    B = rng.standard_normal((Bl + Bu + 1, m)).astype(dt)
    C = rng.standard_normal((Cl + Cu + 1, m)).astype(dt)
    Cd = dev_band(bm, C, n, Cl, Cu, gpu)
    bm.banded_mul_(Cd, dev_band(bm, A, n, Al, Au, gpu), dev_band(bm, B, nu, Bl, Bu, gpu), alpha, beta)
    got = in_matrix(orc, Cd.data.cpu().numpy(), n, Cl, Cu)
    exp = alpha * (in_matrix(orc, A, n, Al, Au).astype(np.float64) @ in_matrix(orc, B, nu, Bl, Bu)) \
        + beta * in_matrix(orc, C, n, Cl, Cu)
    tol = 1e-12 if dt == np.float64 else 2e-5
    assert np.allclose(got, exp, rtol=tol, atol=tol)


def test_gbmm_negative_bands_fill_zero(bm, gpu):
    """test/test_linalg.jl:225-270: negative bandwidths and NaN-filled outputs."""
    rng = np.random.default_rng(4)
    cases = [((2, 2), (-2, 2), (0, 4)), ((-2, 2), (-2, 2), (-4, 4)), ((-2, 2), (2, 2), (0, 4)),
             ((2, 2), (2, -2), (4, 0)), ((2, -2), (2, -2), (4, -4)), ((2, -2), (2, 2), (4, 0))]
    for (al, au), (bl, bu), (cl, cu) in cases:
        A = dev_band(bm, rng.standard_normal((al + au + 1, 10)), 10, al, au, gpu)
        B = dev_band(bm, rng.standard_normal((bl + bu + 1, 10)), 10, bl, bu, gpu)
        C = bm.BandedMatrix(bm.band_storage(cl + cu + 1, 10, torch.float64, gpu, fill=float("nan")), 10, cl, cu)
        bm.banded_mul_(C, A, B)
        exp = (A.to_dense() @ B.to_dense()).cpu().numpy()
        assert np.allclose(C.to_dense().cpu().numpy(), exp, atol=1e-13), ((al, au), (bl, bu))
        bm.banded_mul_(C, A, B, 1.0, 0.0)
        assert np.allclose(C.to_dense().cpu().numpy(), exp, atol=1e-13)
    A = dev_band(bm, rng.standard_normal((1, 1)), 30, 0, 0, gpu)  # 30x1, (0,0)
    B = dev_band(bm, rng.standard_normal((35, 30)), 1, 17, 17, gpu)  # 1x30, (17,17)
    C = bm.BandedMatrix(bm.band_storage(35, 30, torch.float64, gpu, fill=float("nan")), 30, 17, 17)
    bm.banded_mul_(C, A, B)
    assert np.allclose(C.to_dense().cpu().numpy(), (A.to_dense() @ B.to_dense()).cpu().numpy(), atol=1e-13)


def test_gbmm_product_bandwidths_and_star(bm, gpu):
    """A*B allocates bandwidths min(_bnds, prodbandwidths) (test/test_linalg.jl:13-49)."""
    rng = np.random.default_rng(5)
    A = dev_band(bm, rng.standard_normal((4, 10)), 10, 1, 2, gpu)
    C = A @ A
    assert bm.bandwidths(C) == (2, 4)
    assert np.allclose(C.to_dense().cpu().numpy(), (A.to_dense() @ A.to_dense()).cpu().numpy(), atol=1e-13)
    S = dev_band(bm, rng.standard_normal((9, 3)), 3, 4, 4, gpu)
    assert bm.bandwidths(S @ S) == (2, 2)  # clipped to a 3x3 matrix


def test_gbmm_not_enough_bands(bm, gpu):
    """test/test_linalg.jl:272-295: narrower C accepted only when the missing bands are zero."""
    rng = np.random.default_rng(6)
    dA = np.zeros((3, 10))
    dA[1] = rng.standard_normal(10)
    A = dev_band(bm, dA, 10, 1, 1, gpu)  # only the diagonal is nonzero
    B = dev_band(bm, rng.standard_normal((3, 10)), 10, 1, 1, gpu)
    C = bm.BandedMatrix.zeros((10, 10), (1, 1), torch.float64, gpu)
    bm.banded_mul_(C, A, B)
    exp = (A.to_dense() @ B.to_dense()).cpu().numpy()
    assert np.allclose(C.to_dense().cpu().numpy(), exp, atol=1e-14)
    A.data[0, 1:] = torch.from_numpy(rng.standard_normal(9)).to(gpu)
    with pytest.raises(bm.BandError):
        bm.banded_mul_(C, A, B)


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_gbmm_full_size(bm, gpu, orc, dt):
    """n = 2^20, l = u = 16 -> (32,32): bit-exact against the oracle's _gbmm!."""
    n = 1 << 20
    tdt = torch.float64 if dt == np.float64 else torch.float32
    g = torch.Generator(device=gpu)
    g.manual_seed(99)
    A = bm.BandedMatrix(bm.band_storage(33, n, tdt, gpu), n, 16, 16)
    B = bm.BandedMatrix(bm.band_storage(33, n, tdt, gpu), n, 16, 16)
    A.data.uniform_(-1, 1, generator=g)
    B.data.uniform_(-1, 1, generator=g)
    C = bm.banded_mul(A, B)
    assert bm.bandwidths(C) == (32, 32)
    An, Bn = A.data.cpu().numpy(), B.data.cpu().numpy()
    ref = orc.gbmm_percol(n, n, n, 16, 16, 16, 16, 1.0, An, Bn, 0.0, np.zeros((65, n), dtype=dt, order="F"))
    got = C.data.cpu().numpy()
    # in-matrix entries: all but the two 32x32 corner triangles of the storage
    mask = np.ones((65, n), dtype=bool)
    for r in range(65):
        k0 = 32 - r  # column j has matrix row j + r - 32
        if k0 > 0:
            mask[r, :k0] = False
        if r > 32:
            mask[r, n - (r - 32):] = False
    assert np.array_equal(got[mask], ref[mask])


def _dev_band_ld(bm, data_np, m, l, u, device, lda):
    rows, n = data_np.shape
    dt = torch.float64 if data_np.dtype == np.float64 else torch.float32
    d = bm.band_storage(rows, n, dt, device, lda=lda, fill=float("nan"))
    d.copy_(torch.from_numpy(np.ascontiguousarray(data_np)))
    return bm.BandedMatrix(d, m, l, u)


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n,nu,m,Al,Au,Bl,Bu,pad,alpha", [
    (3000, 3000, 3000, 16, 16, 16, 16, 0, 1.0),    # 33 x 33 bands, exact size class
    (3000, 3000, 3000, 4, 3, 4, 3, 0, 1.0),        # the (4,3) x (4,3) product
    (2500, 2600, 2700, 7, 1, 0, 5, 3, 0.75),       # non-square, padded leading dims
    (2900, 2900, 2900, 10, 5, 2, 3, 1, -1.5),      # NA = 16, NB = 6 in the 17 class
    (2100, 2100, 2100, 0, 0, 20, 12, 0, 2.0),      # diagonal times a 33-row band
    (2100, 2100, 2100, 31, 1, 0, 0, 2, 1.0),       # 33-row band times a diagonal
    (1500, 1500, 1500, 8, 8, 8, 8, 0, 0.5),        # 17 x 17, exact
])
def test_gbmm_interior_tiles_bitexact(bm, gpu, orc, dt, n, nu, m, Al, Au, Bl, Bu, pad, alpha):
    """Shapes with interior column tiles (the register-blocked path, beta == 0): every
    in-matrix entry equals the oracle's _gbmm! bit for bit, the edge columns included."""
    rng = np.random.default_rng(n + Al * 7 + Bu)
    A = rng.uniform(-1, 1, (Al + Au + 1, nu)).astype(dt)
    B = rng.uniform(-1, 1, (Bl + Bu + 1, m)).astype(dt)
    A[rng.integers(0, Al + Au + 1, 50), rng.integers(0, nu, 50)] = 0.0
    Ad = _dev_band_ld(bm, A, n, Al, Au, gpu, Al + Au + 1 + pad)
    Bd = _dev_band_ld(bm, B, nu, Bl, Bu, gpu, Bl + Bu + 1 + pad)
    l, u = Al + Bl, Au + Bu
    Cd = _dev_band_ld(bm, np.zeros((l + u + 1, m), dtype=dt), n, l, u, gpu, l + u + 1 + pad)
    Cd.data.fill_(float("nan"))
    bm.banded_mul_(Cd, Ad, Bd, alpha, 0.0)
    ref = orc.gbmm_percol(n, nu, m, Al, Au, Bl, Bu, alpha, A, B, 0.0, np.zeros((l + u + 1, m), dtype=dt, order="F"))
    got = Cd.data.cpu().numpy()
    assert np.array_equal(in_matrix(orc, got, n, l, u), in_matrix(orc, ref, n, l, u))


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_gbmm_interior_wide_c(bm, gpu, orc, dt):
    """C with extra bands on both sides (beta == 0): product rows exact, extra in-matrix
    rows zero, out-of-matrix storage untouched."""
    rng = np.random.default_rng(21)
    n = 2600
    Al, Au, Bl, Bu = 5, 6, 3, 2
    Cl, Cu = Al + Bl + 4, Au + Bu + 3
    A = rng.standard_normal((Al + Au + 1, n)).astype(dt)
    B = rng.standard_normal((Bl + Bu + 1, n)).astype(dt)
    Cd = bm.BandedMatrix(bm.band_storage(Cl + Cu + 1, n, torch.float64 if dt == np.float64 else torch.float32,
                                         gpu, fill=7.0), n, Cl, Cu)
    bm.banded_mul_(Cd, dev_band(bm, A, n, Al, Au, gpu), dev_band(bm, B, n, Bl, Bu, gpu), 1.0, 0.0)
    got = Cd.data.cpu().numpy()
    ref = orc.gbmm_percol(n, n, n, Al, Au, Bl, Bu, 1.0, A, B, 0.0,
                          np.zeros((Al + Bl + Au + Bu + 1, n), dtype=dt, order="F"))
    sh = Cu - (Au + Bu)
    mask = in_matrix(orc, np.ones((Al + Bl + Au + Bu + 1, n)), n, Al + Bl, Au + Bu) != 0
    dref = in_matrix(orc, ref, n, Al + Bl, Au + Bu)
    dgot = in_matrix(orc, got, n, Cl, Cu)
    assert np.array_equal(dgot[mask], dref[mask])
    assert (dgot[~mask] == 0).all()
    for r in range(Cl + Cu + 1):  # storage slots outside the matrix keep their fill
        for j in (0, 1, n - 2, n - 1):
            k = j + r - Cu
            if k < 0 or k >= n:
                assert got[r, j] == 7.0, (r, j)
    assert sh == 3
