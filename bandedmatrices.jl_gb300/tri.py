"""Triangular views of a BandedMatrix and banded x dense products: the reference's
UpperTriangular(A) / LowerTriangular(A) / UnitUpperTriangular(A) / UnitLowerTriangular(A)
with * and \\ (src/tribanded.jl:47-96 -> tbmv!/tbsv!, src/blas.jl:71-147), and
A * B / D * A for a dense B or D (src/generic/matmul.jl:243-271).  Every numerical step
runs in libbandedgpu (bm_{d,s}tbmv, bm_{d,s}tbsv, bm_{d,s}gbmm_bd, bm_{d,s}gbmm_db).
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .banded import BandedMatrix, DimensionMismatch, _prefix, _ptr, _require_cuda, _scalar, _stream


def _colmajor(X: torch.Tensor) -> tuple[torch.Tensor, int]:
    """(column-major tensor with X's values, its leading dimension)."""
    if X.dim() != 2:
        raise ValueError("a matrix is required")
    if X.stride(0) == 1 and (X.shape[1] <= 1 or X.stride(1) >= max(1, X.shape[0])):
        return X, max(1, X.stride(1) if X.shape[1] > 1 else X.shape[0])
    Y = X.t().contiguous().t()
    return Y, max(1, X.shape[0])


def _empty_colmajor(m: int, n: int, like: torch.Tensor) -> torch.Tensor:
    return torch.empty(n, m, dtype=like.dtype, device=like.device).t()


def gbmm_dense_(C: torch.Tensor, A: BandedMatrix, B: torch.Tensor, alpha: float = 1.0, beta: float = 0.0):
    """mul!(C, A, B, alpha, beta), A banded (l, u >= 0), B and C dense: one gbmv 'N' per
    column of B (src/generic/matmul.jl:243-256), all columns in one launch."""
    _require_cuda(A.data, B, C)
    m, n = A.shape
    if B.shape[0] != n or C.shape != (m, B.shape[1]):
        raise DimensionMismatch(f"mul!: A is {m}x{n}, B is {tuple(B.shape)}, C is {tuple(C.shape)}")
    if A.l < 0 or A.u < 0:
        from .linalg import mul_
        for c in range(B.shape[1]):
            col = C[:, c].contiguous()
            mul_(col, A, B[:, c].contiguous(), alpha, beta)
            C[:, c] = col
        return C
    Bc, ldb = _colmajor(B)
    Cc, ldc = _colmajor(C)
    T = A.dtype
    _lib.call(f"bm_{_prefix(T)}gbmm_bd", m, n, A.l, A.u, B.shape[1], _scalar(T, alpha), _ptr(A.data), A.lda,
              _ptr(Bc), ldb, _scalar(T, beta), _ptr(Cc), ldc, _stream(A.device))
    if Cc.data_ptr() != C.data_ptr():
        C.copy_(Cc)
    return C


def dense_gbmm_(C: torch.Tensor, D: torch.Tensor, A: BandedMatrix, alpha: float = 1.0, beta: float = 0.0):
    """mul!(C, D, A, alpha, beta), D and C dense, A banded (l, u >= 0): one gbmv 'T' of A
    per row of D (src/generic/matmul.jl:258-271), all rows in one launch."""
    _require_cuda(A.data, D, C)
    m, n = A.shape
    if D.shape[1] != m or C.shape != (D.shape[0], n):
        raise DimensionMismatch(f"mul!: D is {tuple(D.shape)}, A is {m}x{n}, C is {tuple(C.shape)}")
    if A.l < 0 or A.u < 0:
        from .linalg import mul_t_
        for r in range(D.shape[0]):
            row = C[r, :].contiguous()
            mul_t_(row, A, D[r, :].contiguous(), alpha, beta)
            C[r, :] = row
        return C
    Dc, ldd = _colmajor(D)
    Cc, ldc = _colmajor(C)
    T = A.dtype
    _lib.call(f"bm_{_prefix(T)}gbmm_db", m, n, A.l, A.u, D.shape[0], _scalar(T, alpha), _ptr(Dc), ldd, _ptr(A.data),
              A.lda, _scalar(T, beta), _ptr(Cc), ldc, _stream(A.device))
    if Cc.data_ptr() != C.data_ptr():
        C.copy_(Cc)
    return C


class _Triangular:
    """A triangular view of a square BandedMatrix (the upper or lower band part, with
    the diagonal taken as ones when unit).  `.T` is the transposed view."""

    UPLO = "U"
    UNIT = False

    def __init__(self, A: BandedMatrix, trans: bool = False):
        if A.m != A.n:
            raise DimensionMismatch(f"matrix is not square: dimensions are {A.shape}")
        self.A, self.trans = A, trans
        k = A.u if self.UPLO == "U" else A.l
        if k < 0 or (self.UPLO == "U" and A.u < 0) or A.data.shape[0] < A.l + A.u + 1:
            raise ValueError("triangular banded data missing")
        self.k = k

    @property
    def T(self):
        return type(self)(self.A, not self.trans)

    def _band(self):
        # upper: storage rows 0 .. u (diagonal in row u); lower: rows u .. u+l (diagonal first)
        A = self.A
        off = 0 if self.UPLO == "U" else A.u
        return A.data, off

    def _call(self, fn: str, x: torch.Tensor) -> torch.Tensor:
        _require_cuda(self.A.data, x)
        n = self.A.n
        if x.dim() != 1 or x.shape[0] != n:
            raise DimensionMismatch(f"size of A is {n} != length(x) = {tuple(x.shape)}")
        if n == 0:
            return x
        data, off = self._band()
        inc = x.stride(0) if n > 1 else 1
        _lib.call(f"bm_{_prefix(self.A.dtype)}{fn}", self.UPLO.encode(), b"T" if self.trans else b"N",
                  b"U" if self.UNIT else b"N", n, self.k, _ptr(data, off), self.A.lda, _ptr(x), inc,
                  _stream(self.A.device))
        return x

    def lmul_(self, x: torch.Tensor) -> torch.Tensor:
        """lmul!(L, x): x <- op(L) x in place (tbmv!)."""
        return self._call("tbmv", x)

    def ldiv_(self, x: torch.Tensor) -> torch.Tensor:
        """ldiv!(L, x): x <- op(L) \\ x in place (tbsv!)."""
        return self._call("tbsv", x)

    def __matmul__(self, x: torch.Tensor) -> torch.Tensor:
        return self.lmul_(x.clone())

    def solve(self, b: torch.Tensor) -> torch.Tensor:
        return self.ldiv_(b.clone())


class UpperTriangular(_Triangular):
    UPLO, UNIT = "U", False


class LowerTriangular(_Triangular):
    UPLO, UNIT = "L", False


class UnitUpperTriangular(_Triangular):
    UPLO, UNIT = "U", True


class UnitLowerTriangular(_Triangular):
    UPLO, UNIT = "L", True
