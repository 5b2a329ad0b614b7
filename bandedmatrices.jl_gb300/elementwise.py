"""Banded elementwise algebra on device BandedMatrix objects: axpy!(a, X, Y)
(banded_axpy!, src/banded/BandedMatrix.jl:1006-1015 and banded_generic_axpy!,
src/generic/broadcast.jl:978-1020), A + B, A - B, -A, alpha * A (banded_lmul!,
src/generic/broadcast.jl:960-965), A + sigma*I, and dot(x, A, y) (src/banded/dot.jl).
The arithmetic runs in libbandedgpu (bm_{d,s}gbaxpy / gbscal / gbshift / gbdot).
"""
from __future__ import annotations

import torch

from . import _lib
from .banded import BandedMatrix, BandError, DimensionMismatch, _prefix, _ptr, _require_cuda, _scalar, _stream


def axpy_(a: float, X: BandedMatrix, Y: BandedMatrix) -> BandedMatrix:
    """axpy!(a, X, Y): Y <- a X + Y; raises BandError (Y unchanged) when X has a nonzero
    in-matrix entry outside Y's bands, as banded_generic_axpy! does."""
    _require_cuda(X.data, Y.data)
    if X.shape != Y.shape:
        raise DimensionMismatch(f"X has size {X.shape} but Y has size {Y.shape}")
    if X.dtype != Y.dtype:
        raise TypeError("X and Y must have the same element type")
    m, n = X.shape
    bad = torch.empty(1, dtype=torch.int64, device=X.device)
    T = X.dtype
    _lib.call(f"bm_{_prefix(T)}gbaxpy", m, n, _scalar(T, a), X.l, X.u, _ptr(X.data), X.lda, Y.l, Y.u, _ptr(Y.data),
              Y.lda, _ptr(bad), _stream(X.device))
    if (X.l > Y.l or X.u > Y.u) and (X.l, X.u) != (Y.l, Y.u):
        v = int(bad.item()) & 0xFFFFFFFFFFFFFFFF  # reading the flag synchronises, as the reference's check does
        if v != 0xFFFFFFFFFFFFFFFF:
            j, k = divmod(v, m)
            raise BandError(f"attempt to access {m}x{n} BandedMatrix with bandwidths ({Y.l}, {Y.u}) at band {j - k}"
                            f" (entry ({k}, {j}))")
    return Y


def scale_(alpha: float, A: BandedMatrix) -> BandedMatrix:
    """lmul!(alpha, A) on the band storage."""
    _require_cuda(A.data)
    T = A.dtype
    _lib.call(f"bm_{_prefix(T)}gbscal", A.m, A.n, A.l, A.u, _scalar(T, alpha), _ptr(A.data), A.lda,
              _stream(A.device))
    return A


def shift_(A: BandedMatrix, sigma: float) -> BandedMatrix:
    """A <- A + sigma I in place (l, u >= 0)."""
    _require_cuda(A.data)
    T = A.dtype
    _lib.call(f"bm_{_prefix(T)}gbshift", A.m, A.n, A.l, A.u, _scalar(T, sigma), _ptr(A.data), A.lda,
              _stream(A.device))
    return A


def add(A: BandedMatrix, B: BandedMatrix, beta: float = 1.0) -> BandedMatrix:
    """A + beta*B into a new BandedMatrix with bandwidths (max l, max u), as the
    reference's broadcast allocates it."""
    if A.shape != B.shape:
        raise DimensionMismatch(f"sizes {A.shape} and {B.shape} do not match")
    R = BandedMatrix.zeros(A.shape, (max(A.l, B.l), max(A.u, B.u)), A.dtype, A.device)
    axpy_(1.0, A, R)
    axpy_(beta, B, R)
    return R


def dot(x: torch.Tensor, A: BandedMatrix, y: torch.Tensor) -> torch.Tensor:
    """dot(x, A, y) = x' A y as a 0-d device tensor (l, u >= 0)."""
    _require_cuda(A.data, x, y)
    m, n = A.shape
    if x.shape != (m,) or y.shape != (n,):
        raise DimensionMismatch()
    out = torch.empty(1, dtype=A.dtype, device=A.device)
    work = torch.empty(1024, dtype=A.dtype, device=A.device)
    _lib.call(f"bm_{_prefix(A.dtype)}gbdot", m, n, A.l, A.u, _ptr(x.contiguous()), _ptr(A.data), A.lda,
              _ptr(y.contiguous()), _ptr(out), _ptr(work), _stream(A.device))
    return out[0]
