"""CPU oracle for the banded hot path -- TEST INFRASTRUCTURE ONLY.

This package is the checker the CUDA library is compared against.  It is
loaded only by ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py``; the product path (``bandedmatrices.jl_gb300``) never
imports it.

``oracle.c`` restates, in plain C:
  * reference BLAS/LAPACK routines that BandedMatrices.jl ccalls
    (``dgbmv`` src/blas.jl:19-26 and src/generic/matmul.jl:22, ``dgbtrf``
    src/banded/BandedLU.jl:98, ``dgbtrs`` src/banded/linalg.jl:28,46,
    ``dtbsv`` src/blas.jl:134, ``dtbmv`` src/blas.jl:94);
  * the reference's own Julia loops ``_gbmm!`` (src/banded/gbmm.jl:296-340),
    ``banded_mul!`` (src/generic/matmul.jl:143-172), ``_banded_qr!``
    (src/banded/bandedqr.jl:13-28) and ``banded_qr_lmul!``
    (src/banded/bandedqr.jl:38-94).

Band arrays are numpy arrays of shape ``(lda, n)`` in Fortran (column-major)
order, i.e. exactly LAPACK band storage; ``ipiv`` is int64 and 1-based.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "oracle.c")
_LIB = os.path.join(_HERE, "liboracle.so")

CFLAGS = ["-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared"]


def build(force: bool = False) -> str:
    """Compile ``oracle.c`` into ``liboracle.so`` beside it (gcc)."""
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
        tmp = _LIB + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", *CFLAGS, "-o", tmp, _SRC, "-lm"])
        os.replace(tmp, _LIB)
    return _LIB


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB)
        i64, P, c = ctypes.c_int64, ctypes.c_void_p, ctypes.c_char
        for p, T in (("d", ctypes.c_double), ("s", ctypes.c_float)):
            getattr(L, f"or_{p}gbmv").argtypes = [c, i64, i64, i64, i64, T, P, i64, P, i64, T, P, i64]
            getattr(L, f"or_{p}gbtf2").argtypes = [i64, i64, i64, i64, P, i64, P, P]
            getattr(L, f"or_{p}tbsv").argtypes = [c, c, c, i64, i64, P, i64, P]
            getattr(L, f"or_{p}tbmv").argtypes = [c, c, c, i64, i64, P, i64, P]
            getattr(L, f"or_{p}pbtf2").argtypes = [c, i64, i64, P, i64, P]
            getattr(L, f"or_{p}pbtrs").argtypes = [c, i64, i64, i64, P, i64, P, i64]
            getattr(L, f"or_{p}sbmv").argtypes = [c, i64, i64, T, P, i64, P, T, P]
            getattr(L, f"or_{p}gbtrs").argtypes = [c, i64, i64, i64, i64, P, i64, P, P, i64]
            getattr(L, f"or_{p}gbmm_generic").argtypes = [i64] * 9 + [T, P, i64, P, i64, T, P, i64]
            getattr(L, f"or_{p}gbmm_percol").argtypes = [i64] * 7 + [T, P, i64, P, i64, T, P, i64]
            getattr(L, f"or_{p}gbqrf").argtypes = [i64, i64, i64, i64, P, i64, P]
            getattr(L, f"or_{p}gbqr_lmul").argtypes = [c, i64, i64, i64, i64, P, i64, P, i64, i64, P, i64]
            getattr(L, f"or_{p}gbmm_percol_cblas").argtypes = [P] + [i64] * 7 + [T, P, i64, P, i64, T, P, i64]
        L.or_dgb_adjoint.argtypes = [i64, i64, i64, P, i64, P, P, P, P, P, i64]
        _lib = L
    return _lib


def _pfx(a: np.ndarray) -> str:
    if a.dtype == np.float64:
        return "d"
    if a.dtype == np.float32:
        return "s"
    raise TypeError(f"oracle: unsupported dtype {a.dtype}")


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def _fortran(a: np.ndarray, dtype=None) -> np.ndarray:
    return np.array(a, dtype=dtype or a.dtype, order="F", copy=True)


def _check(st: int, name: str) -> None:
    if st != 0:
        raise ValueError(f"oracle {name}: illegal argument {-st}")


def gbmv(trans, m, n, kl, ku, alpha, A, x, beta=0.0, y=None, incx=1, incy=1):
    """y <- alpha*op(A)*x + beta*y (xGBMV); returns a new array."""
    A = np.asfortranarray(A)
    p = _pfx(A)
    T = A.dtype.type
    leny = m if trans in "Nn" else n
    x = np.ascontiguousarray(x, dtype=A.dtype)
    if y is None:
        y = np.zeros(1 + (leny - 1) * abs(incy) if leny > 0 else 0, dtype=A.dtype)
    else:
        y = np.array(y, dtype=A.dtype, copy=True)
    st = getattr(lib(), f"or_{p}gbmv")(trans.encode(), m, n, kl, ku, T(alpha), _ptr(A), A.shape[0],
                                       _ptr(x), incx, T(beta), _ptr(y), incy)
    _check(st, "gbmv")
    return y


def gbtf2(m, n, kl, ku, AB):
    """Unblocked xGBTF2 on a copy of AB ((2kl+ku+1) x n storage).  Returns (LU, ipiv, info)."""
    LU = _fortran(AB)
    p = _pfx(LU)
    ipiv = np.zeros(max(0, min(m, n)), dtype=np.int64)
    info = ctypes.c_int64(0)
    st = getattr(lib(), f"or_{p}gbtf2")(m, n, kl, ku, _ptr(LU), LU.shape[0], _ptr(ipiv), ctypes.byref(info))
    _check(st, "gbtf2")
    return LU, ipiv, int(info.value)


def gbtrs(trans, n, kl, ku, LU, ipiv, B):
    """xGBTRS; B is (n,) or (n, nrhs).  Returns the solution (new array)."""
    LU = np.asfortranarray(LU)
    p = _pfx(LU)
    vec = B.ndim == 1
    X = _fortran(B.reshape(n, -1), LU.dtype)
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int64)
    st = getattr(lib(), f"or_{p}gbtrs")(trans.encode(), n, kl, ku, X.shape[1], _ptr(LU), LU.shape[0],
                                        _ptr(ipiv), _ptr(X), max(1, n))
    _check(st, "gbtrs")
    return X[:, 0].copy() if vec else X


def tbsv(uplo, trans, diag, n, k, A, x):
    A = np.asfortranarray(A)
    p = _pfx(A)
    x = np.array(x, dtype=A.dtype, copy=True)
    st = getattr(lib(), f"or_{p}tbsv")(uplo.encode(), trans.encode(), diag.encode(), n, k, _ptr(A), A.shape[0], _ptr(x))
    _check(st, "tbsv")
    return x


def tbmv(uplo, trans, diag, n, k, A, x):
    """x <- op(A) x for a triangular band (xTBMV); returns a new array."""
    A = np.asfortranarray(A)
    p = _pfx(A)
    x = np.array(x, dtype=A.dtype, copy=True)
    st = getattr(lib(), f"or_{p}tbmv")(uplo.encode(), trans.encode(), diag.encode(), n, k, _ptr(A), A.shape[0], _ptr(x))
    _check(st, "tbmv")
    return x


def pbtf2(uplo, n, kd, AB):
    """Unblocked banded Cholesky (xPBTF2) on a copy of AB ((kd+1) x n symmetric band
    storage).  Returns (factor, info)."""
    F = _fortran(AB)
    p = _pfx(F)
    info = ctypes.c_int64(0)
    st = getattr(lib(), f"or_{p}pbtf2")(uplo.encode(), n, kd, _ptr(F), F.shape[0], ctypes.byref(info))
    _check(st, "pbtf2")
    return F, int(info.value)


def pbtrs(uplo, n, kd, F, B):
    """xPBTRS with the Cholesky factor F; B is (n,) or (n, nrhs).  Returns the solution."""
    F = np.asfortranarray(F)
    p = _pfx(F)
    vec = B.ndim == 1
    X = _fortran(B.reshape(n, -1), F.dtype)
    st = getattr(lib(), f"or_{p}pbtrs")(uplo.encode(), n, kd, X.shape[1], _ptr(F), F.shape[0], _ptr(X), max(1, n))
    _check(st, "pbtrs")
    return X[:, 0].copy() if vec else X


def sbmv(uplo, n, k, alpha, A, x, beta=0.0, y=None):
    """y <- alpha A x + beta y for a symmetric band A ((k+1) x n, xSBMV); returns a new array."""
    A = np.asfortranarray(A)
    p = _pfx(A)
    T = A.dtype.type
    x = np.ascontiguousarray(x, dtype=A.dtype)
    y = np.zeros(n, dtype=A.dtype) if y is None else np.array(y, dtype=A.dtype, copy=True)
    st = getattr(lib(), f"or_{p}sbmv")(uplo.encode(), n, k, T(alpha), _ptr(A), A.shape[0], _ptr(x), T(beta), _ptr(y))
    _check(st, "sbmv")
    return y


def gbmm_generic(n, nu, m, Al, Au, Bl, Bu, Cl, Cu, alpha, A, B, beta, C):
    A, B = np.asfortranarray(A), np.asfortranarray(B)
    C = _fortran(C)
    p = _pfx(A)
    T = A.dtype.type
    st = getattr(lib(), f"or_{p}gbmm_generic")(n, nu, m, Al, Au, Bl, Bu, Cl, Cu, T(alpha), _ptr(A), A.shape[0],
                                               _ptr(B), B.shape[0], T(beta), _ptr(C), C.shape[0])
    _check(st, "gbmm_generic")
    return C


def gbmm_percol(n, nu, m, Al, Au, Bl, Bu, alpha, A, B, beta, C):
    """_gbmm! restatement; C must have exactly (Al+Bl, Au+Bu) bands."""
    A, B = np.asfortranarray(A), np.asfortranarray(B)
    C = _fortran(C)
    p = _pfx(A)
    T = A.dtype.type
    st = getattr(lib(), f"or_{p}gbmm_percol")(n, nu, m, Al, Au, Bl, Bu, T(alpha), _ptr(A), A.shape[0],
                                              _ptr(B), B.shape[0], T(beta), _ptr(C), C.shape[0])
    _check(st, "gbmm_percol")
    return C


def gbqrf(m, n, l, u, D):
    """_banded_qr! on a copy of D (bandwidths (l, u), u already padded).  Returns (factors, tau)."""
    F = _fortran(D)
    p = _pfx(F)
    tau = np.zeros(min(m, n), dtype=F.dtype)
    st = getattr(lib(), f"or_{p}gbqrf")(m, n, l, u, _ptr(F), F.shape[0], _ptr(tau))
    _check(st, "gbqrf")
    return F, tau


def gbqr_lmul(trans, m, n, l, u, F, tau, B):
    F = np.asfortranarray(F)
    p = _pfx(F)
    vec = B.ndim == 1
    X = _fortran(B.reshape(m, -1), F.dtype)
    tau = np.ascontiguousarray(tau, dtype=F.dtype)
    st = getattr(lib(), f"or_{p}gbqr_lmul")(trans.encode(), m, n, l, u, _ptr(F), F.shape[0], _ptr(tau), len(tau),
                                            X.shape[1], _ptr(X), max(1, m))
    _check(st, "gbqr_lmul")
    return X[:, 0].copy() if vec else X


def gb_adjoint(n, kl, ku, LU, ipiv, x, w):
    """(dL/db, dL/dband) for L = w.x, x = A\\b, from the factors of A (band gradient in BLAS storage)."""
    LU = np.asfortranarray(LU, dtype=np.float64)
    gb = np.zeros(n)
    gband = np.zeros((kl + ku + 1, n), order="F")
    st = lib().or_dgb_adjoint(n, kl, ku, _ptr(LU), LU.shape[0], _ptr(np.ascontiguousarray(ipiv, dtype=np.int64)),
                              _ptr(np.ascontiguousarray(x, dtype=np.float64)), _ptr(np.ascontiguousarray(w, dtype=np.float64)),
                              _ptr(gb), _ptr(gband), kl + ku + 1)
    _check(st, "gb_adjoint")
    return gb, gband


# ---------------------------------------------------------------------------
# numpy helpers: band storage <-> dense, the storage layouts the reference uses
# ---------------------------------------------------------------------------

def band_to_dense(data: np.ndarray, m: int, l: int, u: int) -> np.ndarray:
    """Dense m x n copy of a BandedMatrix's (l+u+1) x n data (inbands_getindex,
    src/banded/BandedMatrix.jl:414-419: A[k,j] = data[u+k-j+1, j])."""
    n = data.shape[1]
    A = np.zeros((m, n), dtype=data.dtype)
    for j in range(n):
        for k in range(max(0, j - u), min(m, j + l + 1)):
            A[k, j] = data[u + k - j, j]
    return A


def dense_to_band(A: np.ndarray, l: int, u: int, lda: int | None = None, row0: int = 0) -> np.ndarray:
    """Band storage of A with bandwidths (l,u); rows [row0, row0+l+u+1) of an lda-row array
    (row0 = l for the gbtrf layout whose top l rows hold the fill-in).  Off-matrix slots are 0."""
    m, n = A.shape
    lda = lda or (l + u + 1 + row0)
    D = np.zeros((lda, n), dtype=A.dtype, order="F")
    for j in range(n):
        for k in range(max(0, j - u), min(m, j + l + 1)):
            D[row0 + u + k - j, j] = A[k, j]
    return D


def lu_storage(data: np.ndarray, m: int, l: int, u: int) -> np.ndarray:
    """The (2l+u+1) x n gbtrf input that _lu builds (src/banded/BandedLU.jl:108-111): the band
    re-widened to (l, l+u), extra top rows zero."""
    n = data.shape[1]
    AB = np.zeros((2 * l + u + 1, n), dtype=data.dtype, order="F")
    AB[l:, :] = data
    return AB


def backward_error(A_dense: np.ndarray, x: np.ndarray, b: np.ndarray) -> float:
    """Normwise relative backward error ||Ax-b||_inf / (||A||_inf ||x||_inf + ||b||_inf)."""
    r = A_dense @ x - b
    den = np.abs(A_dense).sum(axis=1).max() * np.abs(x).max() + np.abs(b).max()
    return float(np.abs(r).max() / den) if den > 0 else float(np.abs(r).max())
