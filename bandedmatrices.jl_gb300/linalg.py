"""The reference's linear-algebra surface on device BandedMatrix objects:
``*``/``mul!`` (src/generic/matmul.jl), ``\\``/``ldiv!``/``lu`` (src/banded/BandedLU.jl,
src/banded/linalg.jl) and ``qr`` (src/banded/bandedqr.jl).  Every numerical
step runs in libbandedgpu; this module only does the host-side dispatch the
Julia code does (views for negative bandwidths, result allocation, checks).
"""
from __future__ import annotations

import torch

from . import _lib
from .banded import BandedMatrix, DimensionMismatch, _require_cuda, gbmv


def _fill_rmul_(y: torch.Tensor, beta: float) -> None:
    """_fill_rmul! (src/generic/utils.jl:30): y *= beta, or zero when beta == 0."""
    if beta == 0:
        y.zero_()
    elif beta != 1:
        y.mul_(beta)


def mul_(y: torch.Tensor, A: BandedMatrix, x: torch.Tensor, alpha: float = 1.0, beta: float = 0.0) -> torch.Tensor:
    """mul!(y, A, x, alpha, beta) for a vector x: materialize! (src/generic/matmul.jl:61-64)
    -> _banded_muladd! (:41-59), which views A so that the BLAS sees non-negative
    bandwidths -> _banded_gbmv! (:26-39) -> gbmv."""
    _require_cuda(A.data, x, y)
    m, n = A.shape
    if x.shape != (n,) or y.shape != (m,):
        raise DimensionMismatch(f"mul!: A is {m}x{n}, x has {tuple(x.shape)}, y has {tuple(y.shape)}")
    l, u = A.l, A.u
    if y.numel() == 0:
        return y
    if -l > u or x.numel() == 0:
        _fill_rmul_(y, beta)
        return y
    if l < 0:
        # view(A, :, 1-l:n): columns shifted by -l, bandwidths (0, u+l)
        c = -l
        if c >= n:
            _fill_rmul_(y, beta)
            return y
        V = BandedMatrix(A.data[:, c:], m, 0, u + l)
        gbmv("N", alpha, V, x[c:], beta, y)
        return y
    if u < 0:
        # view(A, 1-u:m, :): rows shifted by -u, bandwidths (l+u, 0)
        r = -u
        _fill_rmul_(y[:r], beta)
        if r >= m:
            return y
        V = BandedMatrix(A.data, m - r, l + u, 0)
        gbmv("N", alpha, V, x, beta, y[r:])
        return y
    gbmv("N", alpha, A, x, beta, y)
    return y


def mul_t_(y: torch.Tensor, A: BandedMatrix, x: torch.Tensor, alpha: float = 1.0, beta: float = 0.0) -> torch.Tensor:
    """mul!(y, transpose(A), x, alpha, beta): the 'T' gbmv path (src/generic/matmul.jl:66-86)."""
    _require_cuda(A.data, x, y)
    m, n = A.shape
    if x.shape != (m,) or y.shape != (n,):
        raise DimensionMismatch(f"mul!: A' is {n}x{m}, x has {tuple(x.shape)}, y has {tuple(y.shape)}")
    l, u = A.l, A.u
    if y.numel() == 0:
        return y
    if -l > u or x.numel() == 0:
        _fill_rmul_(y, beta)
        return y
    if l < 0:
        c = -l
        _fill_rmul_(y[:c], beta)
        if c >= n:
            return y
        V = BandedMatrix(A.data[:, c:], m, 0, u + l)
        gbmv("T", alpha, V, x, beta, y[c:])
        return y
    if u < 0:
        r = -u
        if r >= m:
            _fill_rmul_(y, beta)
            return y
        V = BandedMatrix(A.data, m - r, l + u, 0)
        gbmv("T", alpha, V, x[r:], beta, y)
        return y
    gbmv("T", alpha, A, x, beta, y)
    return y


def mul(A: BandedMatrix, X):
    """A * x (vector) or A * B (BandedMatrix): allocates the result like similar(::MulAdd)
    (src/generic/matmul.jl:1-14) and fills it with mul!."""
    if isinstance(X, BandedMatrix):
        from .gbmm import banded_mul
        return banded_mul(A, X)
    if X.dim() == 1:
        y = torch.empty(A.m, dtype=A.dtype, device=A.device)
        return mul_(y, A, X, 1.0, 0.0)
    if X.dim() == 2:
        from .tri import _empty_colmajor, gbmm_dense_
        return gbmm_dense_(_empty_colmajor(A.m, X.shape[1], X), A, X, 1.0, 0.0)
    raise TypeError("unsupported operand")


def ldiv(A: BandedMatrix, b):
    """A \\ b: square -> lu, otherwise qr (_factorize, src/banded/linalg.jl:75)."""
    if A.m == A.n:
        from .lu import lu
        return lu(A).solve(b)
    from .qr import qr
    return qr(A).solve(b)
