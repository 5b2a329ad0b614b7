"""Generate tests/golden/lapack_golden.npz: golden input/output vectors for the banded path.

BandedMatrices.jl delegates the arithmetic of this path to OpenBLAS (dgbmv_,
dgbtrf_, dgbtrs_, dtbsv_ through ccall, src/blas.jl and src/banded/*.jl) and
ships no golden vectors of its own.  Julia is not installed here, so these
vectors come from the same library routines as SciPy bundles them (OpenBLAS
0.3.x, reference LAPACK algorithms), driven exactly as the reference drives
them:
  * gbmv:   dgbmv on the (l+u+1) x n data        (banded_gbmv!, matmul.jl:21-23)
  * lu:     dgbtrf(l, u, data widened to (l,l+u)) (lu!, BandedLU.jl:90-103, _lu :108-111)
  * solve:  dgbtrs 'N' and 'T'                   (ldiv!, linalg.jl:24-30, :41-47)
  * gbmm:   the _gbmm! column loop, one dgbmv per column (gbmm.jl:296-340)
  * tbsv:   dtbsv upper                           (tbsv!, blas.jl:112-147)
  * qr:     dense dgeqrf on Matrix(A), whose Householder convention equals
            reflector! (the reference pins qr(A).factors/.tau to the unblocked
            dense QR, test/test_bandedqr.jl:34-36)
Inputs are NumPy PCG64 streams and are stored beside the outputs.

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import glob
import os

import numpy as np
import scipy
from scipy.linalg import blas, lapack

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lapack_golden.npz")


def lu_storage(data, l, u):
    n = data.shape[1]
    AB = np.zeros((2 * l + u + 1, n), order="F")
    AB[l:, :] = data
    return AB


def band_to_dense(data, m, l, u):
    n = data.shape[1]
    A = np.zeros((m, n), dtype=data.dtype)
    for j in range(n):
        for k in range(max(0, j - u), min(m, j + l + 1)):
            A[k, j] = data[u + k - j, j]
    return A


def _openblas():
    """SciPy's bundled OpenBLAS (LP64).  Its dgbmv is called through CBLAS because the
    f2py wrapper rejects m < kl+ku+1, which the _gbmm! column windows produce."""
    libdir = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    L = ctypes.CDLL(glob.glob(os.path.join(libdir, "libscipy_openblas*.so"))[0])
    i, d, p = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
    L.scipy_cblas_dgbmv.argtypes = [i, i, i, i, i, i, d, p, i, p, i, d, p, i]
    L.scipy_cblas_dgbmv.restype = None
    return L


_OB = None


def cblas_dgbmv_ptr(m, n, kl, ku, alpha, a, aoff, lda, x, xoff, beta, y, yoff):
    """dgbmv on raw storage with element offsets (the pointer form of src/blas.jl:16-28)."""
    global _OB
    if _OB is None:
        _OB = _openblas()
    ptr = lambda arr, off: ctypes.c_void_p(arr.ctypes.data + off * arr.itemsize)
    _OB.scipy_cblas_dgbmv(102, 111, m, n, kl, ku, alpha, ptr(a, aoff), lda, ptr(x, xoff), 1, beta, ptr(y, yoff), 1)


def gbmm_percol_scipy(n, nu, m, Al, Au, Bl, Bu, alpha, A, B, beta, C):
    """_gbmm! (gbmm.jl:296-340) with SciPy's dgbmv for each column; C has (Al+Bl, Au+Bu) bands."""
    Cl, Cu = Al + Bl, Au + Bu
    a = np.asfortranarray(A).ravel(order="F")
    b = np.asfortranarray(B).ravel(order="F")
    c = np.asfortranarray(C).ravel(order="F").copy()
    sta, stb, stc = A.shape[0], B.shape[0], C.shape[0]

    def gbmv(mm, nn, kl, ku, aoff, boff, coff):
        if mm <= 0 or nn <= 0:
            return
        cblas_dgbmv_ptr(mm, nn, kl, ku, alpha, a, aoff, sta, b, boff, beta, c, coff)

    for j in range(1, min(m, 1 + Bu) + 1):
        gbmv(min(Cl + j, n), min(Bl + j, nu), Al, Au, 0, (j - 1) * stb + Bu - j + 1, (j - 1) * stc + Cu - j + 1)
    for j in range(2 + Bu, min(1 + Cu, nu + Bu, m) + 1):
        gbmv(min(Cl + j, n), min(Bl + Bu + 1, nu - j + Bu + 1), Al + j - Bu - 1, Au - j + Bu + 1,
             (j - Bu - 1) * sta, (j - 1) * stb, (j - 1) * stc + Cu - j + 1)
    for j in range(2 + Cu, min(m, nu + Bu, n + Cu) + 1):
        gbmv(min(Cl + Cu + 1, n - j + Cu + 1), min(Bl + Bu + 1, nu - (j - Bu) + 1), Al + Au, 0,
             (j - Bu - 1) * sta, (j - 1) * stb, (j - 1) * stc)
    for j in range(nu + Bu + 1, min(m, n + Cu) + 1):
        sl = slice((j - 1) * stc, (j - 1) * stc + Cl + Cu + 1)
        c[sl] = 0.0 if beta == 0 else beta * c[sl]
    return c.reshape(C.shape, order="F")


def main():
    g = {}
    rng = np.random.default_rng(20240601)

    # gbmv: shapes of test/test_banded.jl:97-134 (non-negative bands) plus rectangular
    for t, (m, n, kl, ku, alpha, beta, tr) in enumerate(
            [(50, 50, 2, 3, 1.0, 0.0, 0), (40, 60, 3, 1, 0.7, 1.3, 0), (60, 40, 0, 4, -1.1, 0.0, 1),
             (257, 257, 32, 32, 1.0, 0.5, 0), (257, 257, 32, 32, 2.0, 0.0, 1), (1000, 1000, 1, 1, 1.0, 0.0, 0)]):
        data = rng.standard_normal((kl + ku + 1, n))
        x = rng.standard_normal(n if tr == 0 else m)
        y0 = rng.standard_normal(m if tr == 0 else n)
        y = blas.dgbmv(m, n, kl, ku, alpha, np.asfortranarray(data), x, beta=beta, y=y0.copy(), trans=tr)
        g[f"gbmv{t}_dims"] = np.array([m, n, kl, ku, tr], dtype=np.int64)
        g[f"gbmv{t}_ab"] = np.array([alpha, beta])
        g[f"gbmv{t}_data"], g[f"gbmv{t}_x"], g[f"gbmv{t}_y0"], g[f"gbmv{t}_y"] = data, x, y0, y

    # lu + solves: unshifted randn (pivoting exercised), diagonal-shifted, the 5x5 (1,1)
    # case of test/test_bandedlu.jl:26-38, and one case in dgbtrf's blocked regime
    for t, (n, l, u, shift, nrhs) in enumerate(
            [(5, 1, 1, 0.0, 1), (300, 4, 3, 0.0, 3), (300, 4, 3, 10.0, 1), (200, 30, 2, 0.0, 2),
             (200, 2, 30, 0.0, 1), (257, 33, 70, 0.0, 2), (64, 1, 0, 0.0, 1), (64, 0, 1, 0.0, 1)]):
        data = rng.standard_normal((l + u + 1, n))
        data[u, :] += shift
        AB = lu_storage(data, l, u)
        LU, ipiv, info = lapack.dgbtrf(AB.copy(order="F"), l, u)
        b = rng.standard_normal((n, nrhs))
        xN, _ = lapack.dgbtrs(LU, l, u, b, ipiv, trans=0)
        xT, _ = lapack.dgbtrs(LU, l, u, b, ipiv, trans=1)
        g[f"lu{t}_dims"] = np.array([n, l, u, nrhs, info], dtype=np.int64)
        g[f"lu{t}_data"], g[f"lu{t}_LU"], g[f"lu{t}_ipiv"] = data, LU, (ipiv + 1).astype(np.int64)
        g[f"lu{t}_b"], g[f"lu{t}_xN"], g[f"lu{t}_xT"] = b, xN, xT

    # tbsv upper 'N'/'T'
    for t, (n, k) in enumerate([(100, 3), (80, 20)]):
        Ab = rng.standard_normal((k + 1, n))
        Ab[k, :] += 4.0 * np.sign(Ab[k, :])
        x = rng.standard_normal(n)
        g[f"tbsv{t}_dims"] = np.array([n, k], dtype=np.int64)
        g[f"tbsv{t}_A"], g[f"tbsv{t}_x"] = Ab, x
        g[f"tbsv{t}_yN"] = blas.dtbsv(k, np.asfortranarray(Ab), x.copy(), lower=0, trans=0)
        g[f"tbsv{t}_yT"] = blas.dtbsv(k, np.asfortranarray(Ab), x.copy(), lower=0, trans=1)

    # gbmm via the _gbmm! column loop over dgbmv
    for t, (n, nu, m, Al, Au, Bl, Bu) in enumerate(
            [(50, 50, 50, 2, 1, 1, 2), (50, 5, 50, 30, 2, 1, 30), (5, 50, 50, 0, 30, 2, 1), (40, 40, 40, 4, 3, 4, 3)]):
        A = rng.standard_normal((Al + Au + 1, nu))
        B = rng.standard_normal((Bl + Bu + 1, m))
        C = rng.standard_normal((Al + Bl + Au + Bu + 1, m))
        alpha, beta = 0.123, 0.456
        g[f"gbmm{t}_dims"] = np.array([n, nu, m, Al, Au, Bl, Bu], dtype=np.int64)
        g[f"gbmm{t}_A"], g[f"gbmm{t}_B"], g[f"gbmm{t}_C0"] = A, B, C
        g[f"gbmm{t}_C"] = gbmm_percol_scipy(n, nu, m, Al, Au, Bl, Bu, alpha, A, B, beta, C)

    # qr: shapes of test/test_bandedqr.jl:34-62
    for t, (m, n, l, u) in enumerate([(100, 100, 3, 4), (102, 100, 3, 4), (100, 102, 3, 4), (100, 100, 1, 1),
                                      (10, 10, 3, 2), (14, 10, 3, 2)]):
        data = rng.uniform(0.0, 1.0, (l + u + 1, n))
        A = band_to_dense(data, m, l, u)
        qrf, tau, work, info = lapack.dgeqrf(np.asfortranarray(A))
        b = rng.standard_normal(m)
        g[f"qr{t}_dims"] = np.array([m, n, l, u], dtype=np.int64)
        g[f"qr{t}_data"], g[f"qr{t}_qr"], g[f"qr{t}_tau"], g[f"qr{t}_b"] = data, qrf, tau, b
        if m >= n:
            g[f"qr{t}_x"] = np.linalg.lstsq(A, b, rcond=None)[0]

    # the CPU-runnable case: brandn(10000,10000,4,3) + 10 on the diagonal
    n, l, u = 10000, 4, 3
    r0 = np.random.default_rng(0)
    data = r0.standard_normal((l + u + 1, n))
    data[u, :] += 10.0
    b = r0.standard_normal(n)
    y = blas.dgbmv(n, n, l, u, 1.0, np.asfortranarray(data), b)
    LU, ipiv, info = lapack.dgbtrf(lu_storage(data, l, u), l, u)
    x, _ = lapack.dgbtrs(LU, l, u, b, ipiv)
    AA = gbmm_percol_scipy(n, n, n, l, u, l, u, 1.0, data, data, 0.0, np.zeros((2 * (l + u) + 1, n), order="F"))
    cols = np.sort(np.random.default_rng(1).choice(n, 400, replace=False))
    g["cfg1_data"], g["cfg1_b"], g["cfg1_y"], g["cfg1_x"] = data, b, y, x
    g["cfg1_ipiv"] = (ipiv + 1).astype(np.int32)
    g["cfg1_cols"] = cols.astype(np.int64)
    g["cfg1_LUcols"] = LU[:, cols]
    g["cfg1_AAcols"] = AA[:, cols]

    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1e6:.2f} MB, {len(g)} arrays)")


if __name__ == "__main__":
    main()
