"""Banded Cholesky (bm_{d,s}pbtrf / pbtrs) and the symmetric band product
(bm_{d,s}sbmv) on the GPU against the oracle.

The factorization follows xPBTF2 element for element, so factors equal the oracle's bit
for bit, in both storage halves and both precisions; a matrix that is not positive
definite stops with info at the first failing leading minor, as LAPACK reports it.
xPBTRS is two triangular band sweeps per right-hand side, and xSBMV computes each output
in reference DSBMV's order: both bit for bit.  OpenBLAS itself (the golden file) agrees
to 1e-13 (its dpbtrf is blocked for kd >= 32).  Cases follow
test/test_symbanded.jl's Cholesky checks (factor, solve, a non-positive-definite
matrix).
"""
import ctypes
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
NEXT = os.path.join(os.path.dirname(__file__), "golden", "next_golden.npz")


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _spd(rng, n, k, uplo, dt):
    A = rng.standard_normal((k + 1, n)).astype(dt)
    d = k if uplo == "U" else 0
    A[d] = np.abs(A[d]) + dt(2.0 * (k + 1))
    return A


def _factor(bm, gpu, uplo, A, n, k):
    L = bm._lib.load()
    Ad = torch.from_numpy(np.ascontiguousarray(A.T)).to(gpu)
    info = torch.full((1,), -9, dtype=torch.int64, device=gpu)
    pfx = "d" if A.dtype == np.float64 else "s"
    st = getattr(L, f"bm_{pfx}pbtrf")(uplo.encode(), n, k, ctypes.c_void_p(Ad.data_ptr()), k + 1,
                                      ctypes.c_void_p(info.data_ptr()), _stream())
    assert st == 0, L.bm_last_error()
    return Ad, int(info.item())


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("uplo", ["U", "L"])
@pytest.mark.parametrize("n,k", [(1, 0), (7, 3), (300, 0), (500, 5), (1000, 40), (2000, 128), (400, 167)])
def test_pbtrf_pbtrs_bitexact(bm, gpu, orc, dt, uplo, n, k):
    rng = np.random.default_rng(n + 3 * k)
    A = _spd(rng, n, k, uplo, dt)
    Fd, info = _factor(bm, gpu, uplo, A, n, k)
    F, info_o = orc.pbtf2(uplo, n, k, A)
    assert info == info_o == 0
    got = Fd.cpu().numpy().T
    # the storage slots outside the matrix (the first k columns' top rows for 'U', the
    # last k columns' bottom rows for 'L') are never touched
    assert np.array_equal(got, F), f"factor differs by {np.abs(got - F).max()}"
    B = rng.standard_normal((n, 3)).astype(dt)
    Bd = torch.from_numpy(np.ascontiguousarray(B.T)).to(gpu)
    L = bm._lib.load()
    st = getattr(L, f"bm_{'d' if dt == np.float64 else 's'}pbtrs")(
        uplo.encode(), n, k, 3, ctypes.c_void_p(Fd.data_ptr()), k + 1, ctypes.c_void_p(Bd.data_ptr()), n, _stream())
    assert st == 0, L.bm_last_error()
    assert np.array_equal(Bd.cpu().numpy().T, orc.pbtrs(uplo, n, k, F, B))


@pytest.mark.parametrize("uplo", ["U", "L"])
def test_pbtrf_not_positive_definite(bm, gpu, orc, uplo):
    n, k = 300, 9
    rng = np.random.default_rng(4)
    A = _spd(rng, n, k, uplo, np.float64)
    A[k if uplo == "U" else 0, 123] = -50.0
    _, info = _factor(bm, gpu, uplo, A, n, k)
    _, info_o = orc.pbtf2(uplo, n, k, A)
    assert info == info_o and 0 < info <= 124


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("uplo", ["U", "L"])
@pytest.mark.parametrize("incx,incy", [(1, 1), (2, -1)])
def test_sbmv_bitexact(bm, gpu, orc, dt, uplo, incx, incy):
    n, k = 777, 21
    rng = np.random.default_rng(6)
    A = rng.standard_normal((k + 1, n)).astype(dt)
    x = rng.standard_normal(n).astype(dt)
    y0 = rng.standard_normal(n).astype(dt)
    ref = orc.sbmv(uplo, n, k, 0.75, A, x, -1.25, y0)

    def lay(v, inc):
        buf = np.full(1 + (n - 1) * abs(inc), np.nan, dtype=dt)
        idx = np.arange(n) * abs(inc)
        idx = idx[::-1] if inc < 0 else idx
        buf[idx] = v
        return torch.from_numpy(buf).to(gpu), idx

    xd, _ = lay(x, incx)
    yd, iy = lay(y0, incy)
    Ad = torch.from_numpy(np.ascontiguousarray(A.T)).to(gpu)
    L = bm._lib.load()
    T = ctypes.c_double if dt == np.float64 else ctypes.c_float
    st = getattr(L, f"bm_{'d' if dt == np.float64 else 's'}sbmv")(
        uplo.encode(), n, k, T(0.75), ctypes.c_void_p(Ad.data_ptr()), k + 1, ctypes.c_void_p(xd.data_ptr()), incx,
        T(-1.25), ctypes.c_void_p(yd.data_ptr()), incy, _stream())
    assert st == 0, L.bm_last_error()
    assert np.array_equal(yd.cpu().numpy()[iy], ref)


def test_symmetric_and_cholesky_of_a_banded_matrix(bm, gpu, orc):
    """Symmetric(A) * x and cholesky(Symmetric(A)) \\ b through the host mirror, both halves."""
    n, l, u = 600, 8, 8
    rng = np.random.default_rng(7)
    data = rng.standard_normal((l + u + 1, n))
    data[u] = np.abs(data[u]) + 40.0
    A = bm.BandedMatrix(bm.band_storage(l + u + 1, n, torch.float64, gpu), n, l, u)
    A.data.copy_(torch.from_numpy(data))
    x = rng.standard_normal(n)
    xd = torch.from_numpy(x).to(gpu)
    for uplo, half, k in (("U", data[: u + 1], u), ("L", data[u:], l)):
        S = bm.Symmetric(A, uplo)
        assert np.array_equal((S @ xd).cpu().numpy(), orc.sbmv(uplo, n, k, 1.0, half, x))
        F = bm.cholesky(S)
        assert F.issuccess()
        Fo, _ = orc.pbtf2(uplo, n, k, half)
        assert np.array_equal(F.factors.cpu().numpy(), Fo)
        assert np.array_equal(F.solve(xd).cpu().numpy(), orc.pbtrs(uplo, n, k, Fo, x))


def test_chol_golden(bm, gpu):
    gn = np.load(NEXT)
    for c in range(2):
        n, k = (int(v) for v in gn[f"sym{c}_dims"])
        for uplo in "UL":
            key = f"sym{c}_{uplo}"
            Fd, info = _factor(bm, gpu, uplo, gn[key + "_A"], n, k)
            ref = gn[key + "_F"]
            assert info == 0
            assert np.abs(Fd.cpu().numpy().T - ref).max() <= 1e-13 * np.abs(ref).max()
