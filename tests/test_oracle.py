"""Pins the CPU oracle (the checker of every GPU test) against the reference's numbers.

The reference ships no golden vectors and Julia is not installed, so the pins are
(a) tests/golden/lapack_golden.npz, produced by OpenBLAS (the library the
reference ccalls) driven the way the reference drives it (see make_golden.py),
and (b) the reference's own property tests, restated: dense products
(test/test_linalg.jl:138-222), dense LU/QR conventions (test/test_bandedlu.jl,
test/test_bandedqr.jl:34-36).
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "lapack_golden.npz")


@pytest.fixture(scope="module")
def g():
    return np.load(GOLD)


def _rel(a, b):
    d = np.abs(np.asarray(a) - np.asarray(b)).max() if np.size(a) else 0.0
    s = np.abs(np.asarray(b)).max() if np.size(b) else 1.0
    return d / (s if s > 0 else 1.0)


def test_gbmv_golden(orc, g):
    t = 0
    while f"gbmv{t}_dims" in g:
        m, n, kl, ku, tr = (int(v) for v in g[f"gbmv{t}_dims"])
        alpha, beta = g[f"gbmv{t}_ab"]
        y = orc.gbmv("T" if tr else "N", m, n, kl, ku, alpha, g[f"gbmv{t}_data"], g[f"gbmv{t}_x"], beta, g[f"gbmv{t}_y0"])
        assert _rel(y, g[f"gbmv{t}_y"]) < 1e-14, t
        if not tr:  # the column-oriented 'N' loop is the OpenBLAS order: equal bit for bit
            assert np.array_equal(y, g[f"gbmv{t}_y"]), t
        t += 1
    assert t >= 6


def test_gbtrf_gbtrs_golden(orc, g):
    t = 0
    while f"lu{t}_dims" in g:
        n, l, u, nrhs, info = (int(v) for v in g[f"lu{t}_dims"])
        data = g[f"lu{t}_data"]
        LU, ipiv, inf = orc.gbtf2(n, n, l, u, orc.lu_storage(data, n, l, u))
        assert inf == info
        assert np.array_equal(ipiv, g[f"lu{t}_ipiv"]), f"pivots differ in case {t}"
        blocked = l >= 32 and u > 64  # dgbtrf's blocked regime (ilaenv nb=32)
        if blocked:
            assert _rel(LU[l:], g[f"lu{t}_LU"][l:]) < 1e-12
        else:
            assert np.array_equal(LU[l:], g[f"lu{t}_LU"][l:]), f"unblocked factors differ in case {t}"
        b = g[f"lu{t}_b"]
        xN = orc.gbtrs("N", n, l, u, LU, ipiv, b)
        xT = orc.gbtrs("T", n, l, u, LU, ipiv, b)
        assert _rel(xN, g[f"lu{t}_xN"]) < 1e-12
        assert _rel(xT, g[f"lu{t}_xT"]) < 1e-12
        t += 1
    assert t >= 8


def test_tbsv_golden(orc, g):
    for t in range(2):
        n, k = (int(v) for v in g[f"tbsv{t}_dims"])
        A, x = g[f"tbsv{t}_A"], g[f"tbsv{t}_x"]
        assert _rel(orc.tbsv("U", "N", "N", n, k, A, x), g[f"tbsv{t}_yN"]) < 1e-13
        assert _rel(orc.tbsv("U", "T", "N", n, k, A, x), g[f"tbsv{t}_yT"]) < 1e-13


def test_gbmm_golden(orc, g):
    for t in range(4):
        n, nu, m, Al, Au, Bl, Bu = (int(v) for v in g[f"gbmm{t}_dims"])
        A, B, C0 = g[f"gbmm{t}_A"], g[f"gbmm{t}_B"], g[f"gbmm{t}_C0"]
        Cp = orc.gbmm_percol(n, nu, m, Al, Au, Bl, Bu, 0.123, A, B, 0.456, C0)
        assert np.array_equal(Cp, g[f"gbmm{t}_C"]), t
        Cg = orc.gbmm_generic(n, nu, m, Al, Au, Bl, Bu, Al + Bl, Au + Bu, 0.123, A, B, 0.456, C0)
        # in-matrix entries only: _gbmm! also beta-scales the off-matrix corner slots
        dense = lambda X: orc.band_to_dense(X, n, Al + Bl, Au + Bu)
        assert _rel(dense(Cg), dense(g[f"gbmm{t}_C"])) < 1e-13


def _band_of(orc, F, m, l, u):
    return orc.band_to_dense(F, m, l, u)


def test_qr_golden(orc, g):
    for t in range(6):
        m, n, l, u = (int(v) for v in g[f"qr{t}_dims"])
        data = g[f"qr{t}_data"]
        # _banded_qr pads to (l, l+u) (bandedqr.jl:2)
        D = np.zeros((2 * l + u + 1, n), order="F")
        D[l:, :] = data
        F, tau = orc.gbqrf(m, n, l, l + u, D)
        dense = orc.band_to_dense(F, m, l, l + u)
        mask = orc.band_to_dense(np.ones_like(F), m, l, l + u) != 0
        qr = g[f"qr{t}_qr"]
        assert _rel(dense[mask], qr[mask]) < 1e-12, t
        assert np.abs(qr[~mask]).max(initial=0.0) < 1e-12
        assert _rel(tau, g[f"qr{t}_tau"]) < 1e-12, t
        if f"qr{t}_x" in g:
            b = g[f"qr{t}_b"]
            qtb = orc.gbqr_lmul("T", m, n, l, l + u, F, tau, b)
            # R is the upper band of the factors with bandwidth l+u (tribanded.jl:75-83)
            x = orc.tbsv("U", "N", "N", n, l + u, F, qtb[:n])
            assert _rel(x, g[f"qr{t}_x"]) < 1e-10, t
            qb = orc.gbqr_lmul("N", m, n, l, l + u, F, tau, qtb)
            assert _rel(qb, b) < 1e-13


def test_cpu_runnable_case_golden(orc, g):
    """brandn(10000,10000,4,3) + 10I: A*b, A*A and A\\b against OpenBLAS."""
    data, b = g["cfg1_data"], g["cfg1_b"]
    n, l, u = 10000, 4, 3
    y = orc.gbmv("N", n, n, l, u, 1.0, data, b)
    assert np.array_equal(y, g["cfg1_y"])
    LU, ipiv, info = orc.gbtf2(n, n, l, u, orc.lu_storage(data, n, l, u))
    assert info == 0 and np.array_equal(ipiv, g["cfg1_ipiv"].astype(np.int64))
    cols = g["cfg1_cols"]
    assert np.array_equal(LU[:, cols][l:], g["cfg1_LUcols"][l:])
    x = orc.gbtrs("N", n, l, u, LU, ipiv, b)
    assert _rel(x, g["cfg1_x"]) < 1e-12
    AA = orc.gbmm_percol(n, n, n, l, u, l, u, 1.0, data, data, 0.0, np.zeros((2 * (l + u) + 1, n), order="F"))
    assert np.array_equal(AA[:, cols], g["cfg1_AAcols"])


@pytest.mark.parametrize("n,nu,m", [(1, 1, 1), (1, 5, 50), (5, 5, 5), (50, 5, 1), (5, 50, 50), (50, 50, 50),
                                    (50, 1, 5), (1, 50, 5)])
def test_gbmm_reference_sweep(orc, n, nu, m):
    """test/test_linalg.jl:138-222: every Al,Au,Bl,Bu in {0,1,2,30} against dense alpha*A*B + beta*C."""
    rng = np.random.default_rng(n * 10000 + nu * 100 + m)
    for Al in (0, 1, 2, 30):
        for Au in (0, 1, 2, 30):
            for Bl in (0, 1, 2, 30):
                for Bu in (0, 1, 2, 30):
                    A = rng.uniform(size=(Al + Au + 1, nu))
                    B = rng.uniform(size=(Bl + Bu + 1, m))
                    C = rng.uniform(size=(Al + Bl + Au + Bu + 1, m))
                    Ad = orc.band_to_dense(A, n, Al, Au)
                    Bd = orc.band_to_dense(B, nu, Bl, Bu)
                    Cd = orc.band_to_dense(C, n, Al + Bl, Au + Bu)
                    ex = 0.123 * Ad @ Bd + 0.456 * Cd
                    Cp = orc.gbmm_percol(n, nu, m, Al, Au, Bl, Bu, 0.123, A, B, 0.456, C)
                    Cg = orc.gbmm_generic(n, nu, m, Al, Au, Bl, Bu, Al + Bl, Au + Bu, 0.123, A, B, 0.456, C)
                    assert np.allclose(orc.band_to_dense(Cp, n, Al + Bl, Au + Bu), ex, rtol=1e-13, atol=1e-13)
                    assert np.allclose(orc.band_to_dense(Cg, n, Al + Bl, Au + Bu), ex, rtol=1e-13, atol=1e-13)


def test_lu_pivot_rule_and_dense(orc):
    """Partial pivoting picks the first index of max |a| (idamax); L*U = P*A densely."""
    rng = np.random.default_rng(7)
    for (n, l, u) in [(5, 1, 1), (60, 3, 2), (60, 7, 0), (60, 0, 5)]:
        data = rng.standard_normal((l + u + 1, n))
        data[:, ::7] = np.round(data[:, ::7])  # exact ties
        LU, ipiv, info = orc.gbtf2(n, n, l, u, orc.lu_storage(data, n, l, u))
        A = orc.band_to_dense(data, n, l, u)
        # rebuild P*A = L*U from the band factors
        kv = l + u
        U = np.zeros((n, n))
        L = np.eye(n)
        for j in range(n):
            for i in range(max(0, j - kv), j + 1):
                U[i, j] = LU[kv + i - j, j]
        PA = A.copy()
        Lcols = []
        for j in range(n):
            p = ipiv[j] - 1
            PA[[j, p]] = PA[[p, j]]
            for prev in Lcols:  # apply the row swap to earlier multiplier columns
                prev[[j, p]] = prev[[p, j]]
            col = np.zeros(n)
            for i in range(j + 1, min(n, j + l + 1)):
                col[i] = LU[kv + i - j, j]
            Lcols.append(col)
        for j, col in enumerate(Lcols):
            L[:, j] += col
        assert np.allclose(L @ U, PA, atol=1e-12)


def test_backward_error_small(orc):
    rng = np.random.default_rng(3)
    n, l, u = 400, 6, 5
    data = rng.standard_normal((l + u + 1, n))
    A = orc.band_to_dense(data, n, l, u)
    b = rng.standard_normal(n)
    LU, ipiv, info = orc.gbtf2(n, n, l, u, orc.lu_storage(data, n, l, u))
    x = orc.gbtrs("N", n, l, u, LU, ipiv, b)
    assert orc.backward_error(A, x, b) < 1e-15
    xt = orc.gbtrs("T", n, l, u, LU, ipiv, b)
    assert orc.backward_error(A.T, xt, b) < 1e-15


def test_adjoint_formula(orc):
    """dL/db = A^{-T} w and dL/dA = -(A^{-T} w) x^T on the band, by central differences."""
    rng = np.random.default_rng(11)
    n, l, u = 30, 2, 3
    data = rng.standard_normal((l + u + 1, n))
    data[u] += 5.0
    b, w = rng.standard_normal(n), rng.standard_normal(n)

    def loss(dat, bb):
        LU, ip, _ = orc.gbtf2(n, n, l, u, orc.lu_storage(dat, n, l, u))
        return w @ orc.gbtrs("N", n, l, u, LU, ip, bb)

    LU, ip, _ = orc.gbtf2(n, n, l, u, orc.lu_storage(data, n, l, u))
    x = orc.gbtrs("N", n, l, u, LU, ip, b)
    gb, gband = orc.gb_adjoint(n, l, u, LU, ip, x, w)
    h = 1e-6
    for i in (0, 7, n - 1):
        e = np.zeros(n)
        e[i] = h
        fd = (loss(data, b + e) - loss(data, b - e)) / (2 * h)
        assert abs(fd - gb[i]) < 1e-6 * max(1.0, abs(fd))
    for (r, j) in ((u, 4), (0, 10), (l + u, 3)):
        dp = data.copy(); dp[r, j] += h
        dm = data.copy(); dm[r, j] -= h
        fd = (loss(dp, b) - loss(dm, b)) / (2 * h)
        assert abs(fd - gband[r, j]) < 1e-6 * max(1.0, abs(fd))


BLOCKED = os.path.join(os.path.dirname(__file__), "golden", "blocked_golden.npz")
# normwise factor agreement with OpenBLAS's blocked dgbtrf (dgemm/dtrsm trailing
# updates in another order than dgbtf2's), and solution agreement per case (set by
# each case's conditioning; c5 is a diffusion operator, r512 unshifted random)
BLOCKED_TOL = {"c4a": (1e-12, 1e-11), "c5": (1e-12, 1e-12), "r512": (1e-12, 1e-9)}


@pytest.mark.parametrize("name", ["c4a", "c5", "r512"])
def test_gbtf2_blocked_regime_golden(orc, name):
    """The dgbtf2 restatement against OpenBLAS in its blocked regime (kl >= its block
    size), at the bandwidths of the wide-band workloads: identical pivots, factors and
    solutions within BLOCKED_TOL, backward error <= 1e-12."""
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_blocked_golden as mb

    gb = np.load(BLOCKED)
    data, l, u, b = mb.case_data(name, gb["c5_kfield"])
    n = data.shape[1]
    LU, ipiv, info = orc.gbtf2(n, n, l, u, orc.lu_storage(data, n, l, u))
    assert info == 0
    assert np.array_equal(ipiv, gb[f"{name}_pivoff"].astype(np.int64) + np.arange(1, n + 1))
    cols = gb[f"{name}_cols"]
    ftol, xtol = BLOCKED_TOL[name]
    assert _rel(LU[:, cols], gb[f"{name}_LUcols"]) <= ftol
    x = orc.gbtrs("N", n, l, u, LU, ipiv, b)
    assert _rel(x, gb[f"{name}_x"]) <= xtol
    r = orc.gbmv("N", n, n, l, u, 1.0, data, x) - b
    rowsum = orc.gbmv("N", n, n, l, u, 1.0, np.abs(data), np.ones(n))
    assert np.abs(r).max() / (rowsum.max() * np.abs(x).max() + np.abs(b).max()) <= 1e-12


NEXT = os.path.join(os.path.dirname(__file__), "golden", "next_golden.npz")
TRI_FORMS = [(u, t, d) for u in "UL" for t in "NT" for d in "NU"]


def test_tbmv_tbsv_every_form_golden(orc):
    """The xTBMV / xTBSV restatements against OpenBLAS dtbmv / dtbsv in all eight
    uplo / trans / diag forms (OpenBLAS's kernels may sum in another order: 1e-13)."""
    gn = np.load(NEXT)
    for c in range(2):
        n, k = (int(v) for v in gn[f"tri{c}_dims"])
        for u, t, d in TRI_FORMS:
            key = f"tri{c}_{u}{t}{d}"
            A, x = gn[key + "_A"], gn[key + "_x"]
            assert _rel(orc.tbmv(u, t, d, n, k, A, x), gn[key + "_mv"]) < 1e-13, key
            assert _rel(orc.tbsv(u, t, d, n, k, A, x), gn[key + "_sv"]) < 1e-13, key


def test_banded_dense_products_golden(orc):
    """Banded x dense (a gbmv 'N' per column) and dense x banded (a gbmv 'T' per row)
    against the same loops over OpenBLAS dgbmv."""
    gn = np.load(NEXT)
    for c in range(2):
        m, n, kl, ku, k = (int(v) for v in gn[f"bd{c}_dims"])
        alpha, beta = gn[f"bd{c}_ab"]
        A, B, C0, D, E0 = (gn[f"bd{c}_{s}"] for s in ("A", "B", "C0", "D", "E0"))
        C = np.stack([orc.gbmv("N", m, n, kl, ku, alpha, A, B[:, j], beta, C0[:, j]) for j in range(k)], axis=1)
        E = np.stack([orc.gbmv("T", m, n, kl, ku, alpha, A, D[r, :], beta, E0[r, :]) for r in range(k)], axis=0)
        assert np.array_equal(C, gn[f"bd{c}_C"]), c  # the 'N' loop is OpenBLAS's order
        assert _rel(E, gn[f"bd{c}_E"]) < 1e-14, c


@pytest.mark.parametrize("uplo", ["U", "L"])
def test_pbtf2_pbtrs_sbmv_golden(orc, uplo):
    """The xPBTF2 / xPBTRS / xSBMV restatements against OpenBLAS dpbtrf / dpbtrs / dsbmv
    (kd = 6: OpenBLAS's unblocked path; kd = 40: its blocked dpbtrf, same pivots-free
    result to rounding)."""
    gn = np.load(NEXT)
    for c in range(2):
        n, k = (int(v) for v in gn[f"sym{c}_dims"])
        key = f"sym{c}_{uplo}"
        A = gn[key + "_A"]
        y = orc.sbmv(uplo, n, k, 0.7, A, gn[key + "_x"], -1.5, gn[key + "_y0"])
        assert _rel(y, gn[key + "_sbmv"]) < 1e-14
        F, info = orc.pbtf2(uplo, n, k, A)
        assert info == 0
        assert _rel(F, gn[key + "_F"]) < 1e-13
        X = orc.pbtrs(uplo, n, k, F, gn[key + "_b"])
        assert _rel(X, gn[key + "_X"]) < 1e-13
