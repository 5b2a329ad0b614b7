"""Triangular band solve / product and banded x dense products on the GPU against the
oracle.

bm_{d,s}tbsv and bm_{d,s}tbmv follow reference DTBSV / DTBMV operation by operation, so
every uplo / trans / diag form equals the oracle bit for bit (tests/test_oracle.py pins
the oracle to OpenBLAS); strided and negative increments follow the BLAS convention.
Banded x dense is one gbmv 'N' per column and dense x banded one gbmv 'T' per row
(src/generic/matmul.jl:243-271): both equal the oracle's per-column / per-row gbmv bit
for bit, and OpenBLAS's (the golden file) to 1e-14.  Cases follow test/test_tribanded.jl
(upper/lower, unit/non-unit solves of banded triangular views) and
test/test_banded.jl:140-161 (banded x dense).
"""
import ctypes
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
NEXT = os.path.join(os.path.dirname(__file__), "golden", "next_golden.npz")
FORMS = [(u, t, d) for u in "UL" for t in "NT" for d in "NU"]


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _run(bm, gpu, fn, dt, u, t, d, n, k, A, x, incx=1):
    """bm_{d,s}{fn} on device copies; x laid out with stride incx (BLAS convention)."""
    L = bm._lib.load()
    Ad = torch.from_numpy(np.ascontiguousarray(A.T)).to(gpu)  # (k+1) x n column-major
    m = 1 + (n - 1) * abs(incx)
    buf = np.full(m, np.nan, dtype=A.dtype)
    idx = np.arange(n) * abs(incx)
    if incx < 0:
        idx = idx[::-1]
    buf[idx] = x
    xd = torch.from_numpy(buf).to(gpu)
    st = getattr(L, f"bm_{'d' if dt == np.float64 else 's'}{fn}")(
        u.encode(), t.encode(), d.encode(), n, k, ctypes.c_void_p(Ad.data_ptr()), k + 1,
        ctypes.c_void_p(xd.data_ptr()), incx, _stream())
    assert st == 0, L.bm_last_error()
    out = xd.cpu().numpy()
    return out[idx]


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n,k", [(1, 0), (2, 1), (33, 5), (300, 0), (1000, 40), (257, 70)])
@pytest.mark.parametrize("form", FORMS)
def test_tbsv_tbmv_bitexact(bm, gpu, orc, dt, n, k, form):
    u, t, d = form
    rng = np.random.default_rng(n * 17 + k)
    A = rng.standard_normal((k + 1, n)).astype(dt)
    A[k if u == "U" else 0] += dt(3.0) * np.sign(A[k if u == "U" else 0])
    x = rng.standard_normal(n).astype(dt)
    if n > 3:
        x[n // 3] = 0.0  # the zero-skip of the axpy forms
    for fn in ("tbmv", "tbsv"):
        got = _run(bm, gpu, fn, dt, u, t, d, n, k, A, x)
        ref = getattr(orc, fn)(u, t, d, n, k, A, x)
        assert np.array_equal(got, ref, equal_nan=True), (fn, form)


@pytest.mark.parametrize("incx", [2, -1, -3])
@pytest.mark.parametrize("form", FORMS)
def test_tbsv_tbmv_strided(bm, gpu, orc, incx, form):
    u, t, d = form
    n, k = 200, 9
    rng = np.random.default_rng(5)
    A = rng.standard_normal((k + 1, n))
    A[k if u == "U" else 0] += 3.0
    x = rng.standard_normal(n)
    for fn in ("tbmv", "tbsv"):
        got = _run(bm, gpu, fn, np.float64, u, t, d, n, k, A, x, incx)
        assert np.array_equal(got, getattr(orc, fn)(u, t, d, n, k, A, x)), (fn, incx)


def test_tri_golden(bm, gpu):
    gn = np.load(NEXT)
    for c in range(2):
        n, k = (int(v) for v in gn[f"tri{c}_dims"])
        for u, t, d in FORMS:
            key = f"tri{c}_{u}{t}{d}"
            A, x = gn[key + "_A"], gn[key + "_x"]
            for fn, sfx in (("tbmv", "_mv"), ("tbsv", "_sv")):
                got = _run(bm, gpu, fn, np.float64, u, t, d, n, k, A, x)
                ref = gn[key + sfx]
                assert np.abs(got - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max()), (key, fn)


def test_triangular_views_of_a_banded_matrix(bm, gpu, orc):
    """UpperTriangular(A) \\ b, LowerTriangular(A) * x, unit views and transposes on a
    BandedMatrix with bandwidths (l, u) (test/test_tribanded.jl)."""
    n, l, u = 500, 6, 9
    rng = np.random.default_rng(9)
    data = rng.standard_normal((l + u + 1, n))
    data[u] += 5.0
    A = bm.BandedMatrix(bm.band_storage(l + u + 1, n, torch.float64, gpu), n, l, u)
    A.data.copy_(torch.from_numpy(data))
    b = rng.standard_normal(n)
    bd = torch.from_numpy(b).to(gpu)
    up, lo = data[: u + 1], data[u:]
    cases = [(bm.UpperTriangular(A), "U", "N", "N", up, u), (bm.LowerTriangular(A), "L", "N", "N", lo, l),
             (bm.UnitUpperTriangular(A).T, "U", "T", "U", up, u), (bm.UnitLowerTriangular(A), "L", "N", "U", lo, l),
             (bm.LowerTriangular(A).T, "L", "T", "N", lo, l)]
    for V, uplo, tr, dg, band, k in cases:
        assert np.array_equal(V.solve(bd).cpu().numpy(), orc.tbsv(uplo, tr, dg, n, k, band, b)), (uplo, tr, dg)
        assert np.array_equal((V @ bd).cpu().numpy(), orc.tbmv(uplo, tr, dg, n, k, band, b)), (uplo, tr, dg)


@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
@pytest.mark.parametrize("m,n,l,u,k", [(300, 300, 3, 5, 7), (64, 80, 20, 2, 3), (1000, 1000, 200, 300, 4),
                                       (5, 9, 0, 0, 1), (40, 30, 2, 1, 0)])
def test_banded_dense_products(bm, gpu, orc, dt, m, n, l, u, k):
    """A * B and D * A (test/test_banded.jl:140-161 multiplies 1000x1000 (200,300) by a
    dense matrix), alpha/beta forms through gbmm_dense_ / dense_gbmm_."""
    rng = np.random.default_rng(m + n + l + k)
    nt = np.float64 if dt == torch.float64 else np.float32
    data = rng.standard_normal((l + u + 1, n)).astype(nt)
    A = bm.BandedMatrix(bm.band_storage(l + u + 1, n, dt, gpu), m, l, u)
    A.data.copy_(torch.from_numpy(data))
    B = rng.standard_normal((n, k)).astype(nt)
    D = rng.standard_normal((k, m)).astype(nt)
    C = (A @ torch.from_numpy(B).to(gpu)).cpu().numpy()
    E = (torch.from_numpy(D).to(gpu) @ A).cpu().numpy()
    assert C.shape == (m, k) and E.shape == (k, n)
    if k == 0:
        return
    Cr = np.stack([orc.gbmv("N", m, n, l, u, 1.0, data, B[:, j]) for j in range(k)], axis=1).reshape(m, k)
    Er = np.stack([orc.gbmv("T", m, n, l, u, 1.0, data, D[r, :]) for r in range(k)], axis=0).reshape(k, n)
    assert np.array_equal(C, Cr) and np.array_equal(E, Er)
    alpha, beta = 0.5, -2.0
    C0 = rng.standard_normal((m, k)).astype(nt)
    Cd = torch.from_numpy(C0).to(gpu)
    bm.gbmm_dense_(Cd, A, torch.from_numpy(B).to(gpu), alpha, beta)
    Cr = np.stack([orc.gbmv("N", m, n, l, u, alpha, data, B[:, j], beta, C0[:, j]) for j in range(k)],
                  axis=1).reshape(m, k)
    assert np.array_equal(Cd.cpu().numpy(), Cr)


def test_banded_dense_golden(bm, gpu):
    gn = np.load(NEXT)
    for c in range(2):
        m, n, kl, ku, k = (int(v) for v in gn[f"bd{c}_dims"])
        alpha, beta = (float(v) for v in gn[f"bd{c}_ab"])
        A = bm.BandedMatrix(bm.band_storage(kl + ku + 1, n, torch.float64, gpu), m, kl, ku)
        A.data.copy_(torch.from_numpy(gn[f"bd{c}_A"]))
        C = torch.from_numpy(gn[f"bd{c}_C0"].copy()).to(gpu)
        bm.gbmm_dense_(C, A, torch.from_numpy(gn[f"bd{c}_B"]).to(gpu), alpha, beta)
        assert np.array_equal(C.cpu().numpy(), gn[f"bd{c}_C"])
        E = torch.from_numpy(gn[f"bd{c}_E0"].copy()).to(gpu)
        bm.dense_gbmm_(E, torch.from_numpy(gn[f"bd{c}_D"]).to(gpu), A, alpha, beta)
        ref = gn[f"bd{c}_E"]
        assert np.abs(E.cpu().numpy() - ref).max() <= 1e-14 * np.abs(ref).max()
