"""Symmetric banded matrices: Symmetric(A, uplo) * x (sbmv!, src/blas.jl:35-64) and
cholesky(Symmetric(A)) with its solve (banded_chol!, src/symbanded/BandedCholesky.jl:2-12,
pbtrf!/pbtrs!, src/lapack.jl:268-332).  The symmetric band is the upper (uplo 'U': rows
0..u of A's storage, diagonal in row u) or lower (rows u..u+l, diagonal first) half of a
BandedMatrix's storage; every numerical step runs in libbandedgpu (bm_{d,s}sbmv,
bm_{d,s}pbtrf, bm_{d,s}pbtrs).
"""
from __future__ import annotations

import torch

from . import _lib
from .banded import BandedMatrix, DimensionMismatch, _prefix, _ptr, _require_cuda, _scalar, _stream, band_storage
from .tri import LowerTriangular, UpperTriangular


class Symmetric:
    """Symmetric(A, uplo): A's upper (or lower) band read as a symmetric matrix."""

    def __init__(self, A: BandedMatrix, uplo: str = "U"):
        if A.m != A.n:
            raise DimensionMismatch(f"matrix is not square: dimensions are {A.shape}")
        if uplo not in ("U", "L"):
            raise ValueError("uplo must be 'U' or 'L'")
        self.A, self.uplo = A, uplo
        self.k = A.u if uplo == "U" else A.l
        if self.k < 0:
            raise ValueError("the symmetric half needs a non-negative bandwidth")

    def _band(self):
        return self.A.data, (0 if self.uplo == "U" else self.A.u)

    def mul_(self, y: torch.Tensor, x: torch.Tensor, alpha: float = 1.0, beta: float = 0.0) -> torch.Tensor:
        """mul!(y, Symmetric(A), x, alpha, beta) (xSBMV)."""
        A = self.A
        _require_cuda(A.data, x, y)
        n = A.n
        if x.shape != (n,) or y.shape != (n,):
            raise DimensionMismatch(f"Symmetric(A) is {n}x{n}, x has {tuple(x.shape)}, y has {tuple(y.shape)}")
        if n == 0:
            return y
        data, off = self._band()
        T = A.dtype
        _lib.call(f"bm_{_prefix(T)}sbmv", self.uplo.encode(), n, self.k, _scalar(T, alpha), _ptr(data, off), A.lda,
                  _ptr(x), x.stride(0) if n > 1 else 1, _scalar(T, beta), _ptr(y), y.stride(0) if n > 1 else 1,
                  _stream(A.device))
        return y

    def __matmul__(self, x: torch.Tensor) -> torch.Tensor:
        return self.mul_(torch.empty_like(x), x, 1.0, 0.0)


class BandedCholesky:
    """cholesky(Symmetric(A)): the factor in symmetric band storage ((k+1) x n), A = U'U
    (uplo 'U') or L L' ('L'); info > 0 when the leading minor of that order is not
    positive definite."""

    def __init__(self, factors: torch.Tensor, uplo: str, k: int, info_t: torch.Tensor):
        self.factors, self.uplo, self.k, self.info_t = factors, uplo, k, info_t

    @property
    def info(self) -> int:
        return int(self.info_t.item())

    def issuccess(self) -> bool:
        return self.info == 0

    @property
    def n(self) -> int:
        return int(self.factors.shape[1])

    def _as_banded(self) -> BandedMatrix:
        if self.uplo == "U":
            return BandedMatrix(self.factors, self.n, 0, self.k)
        return BandedMatrix(self.factors, self.n, self.k, 0)

    @property
    def U(self):
        if self.uplo != "U":
            return LowerTriangular(self._as_banded()).T
        return UpperTriangular(self._as_banded())

    @property
    def L(self):
        if self.uplo != "L":
            return UpperTriangular(self._as_banded()).T
        return LowerTriangular(self._as_banded())

    def ldiv_(self, B: torch.Tensor) -> torch.Tensor:
        """ldiv!(F, B): B <- A \\ B in place (xPBTRS); B is (n,) or column-major (n, nrhs)."""
        _require_cuda(self.factors, B)
        n = self.n
        nrhs = 1 if B.dim() == 1 else B.shape[1]
        if B.shape[0] != n:
            raise DimensionMismatch(f"A is {n}x{n}, B has {tuple(B.shape)}")
        ldb = max(1, n) if B.dim() == 1 or nrhs <= 1 else B.stride(1)
        if B.dim() == 2 and nrhs > 1 and B.stride(0) != 1:
            raise ValueError("B must be column-major")
        lda = max(1, self.factors.stride(1)) if n > 1 else self.k + 1
        _lib.call(f"bm_{_prefix(self.factors.dtype)}pbtrs", self.uplo.encode(), n, self.k, nrhs, _ptr(self.factors),
                  lda, _ptr(B), ldb, _stream(self.factors.device))
        return B

    def solve(self, b: torch.Tensor) -> torch.Tensor:
        X = b.clone() if b.dim() == 1 else b.t().contiguous().t()
        return self.ldiv_(X)


def cholesky(S: Symmetric) -> BandedCholesky:
    """cholesky(Symmetric(A)) on a copy of A's symmetric half (banded_chol!, xPBTRF)."""
    A = S.A
    _require_cuda(A.data)
    k, n = S.k, A.n
    data, off = S._band()
    F = band_storage(k + 1, n, A.dtype, A.device)
    F.copy_(data[off: off + k + 1, :])
    info = torch.zeros(1, dtype=torch.int64, device=A.device)
    lda = max(1, F.stride(1)) if n > 1 else k + 1
    _lib.call(f"bm_{_prefix(A.dtype)}pbtrf", S.uplo.encode(), n, k, _ptr(F), lda, _ptr(info), _stream(A.device))
    return BandedCholesky(F, S.uplo, k, info)
