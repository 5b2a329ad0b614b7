"""Banded QR on the device: qr(A), Q / Q' products and qr(A) \\ b.

Mirrors src/banded/bandedqr.jl: ``qr(A)`` copies A into storage widened to
bandwidths (l, l+u) (_banded_qr, :1-2) and factors it in place with Householder
reflectors (_banded_qr!, :13-28, bm_{d,s}gbqrf); ``lmul_(Q', B)`` and
``lmul_(Q, B)`` run banded_qr_lmul! (:38-94, bm_{d,s}gbqr_lmul); ``solve`` follows
ldiv!(::QR) (:186-207): Q'b, then the upper triangular band solve with R
(UpperTriangular(R) \\ b -> tbsv!, src/tribanded.jl:75-83, bm_{d,s}tbsv).
"""
from __future__ import annotations

import torch

from . import _lib
from .banded import BandedMatrix, DimensionMismatch, _prefix, _ptr, _require_cuda, _stream, band_storage


class BandedQR:
    """``factors`` (BandedMatrix with bandwidths (l, l+u)) and ``tau``."""

    def __init__(self, factors: BandedMatrix, tau: torch.Tensor):
        self.factors, self.tau = factors, tau

    @property
    def shape(self):
        return self.factors.shape

    @property
    def Q(self) -> "QRPackedQ":
        return QRPackedQ(self, False)

    @property
    def R(self) -> torch.Tensor:
        """Dense upper triangular R (min(m,n) x n), a device tensor (inspection/tests)."""
        m, n = self.shape
        return torch.triu(self.factors.to_dense()[: min(m, n), :])

    def solve(self, b: torch.Tensor) -> torch.Tensor:
        """qr(A) \\ b for square or tall A (ldiv!(::QR), src/banded/bandedqr.jl:178-207)."""
        m, n = self.shape
        _require_cuda(b)
        if b.shape[0] != m:
            raise DimensionMismatch(f"B has leading dimension {b.shape[0]}, but needs {m}")
        if n > m:
            raise NotImplementedError("qr \\ b for wide matrices is not implemented (as in the reference)")
        vec = b.dim() == 1
        B = b.reshape(m, -1)
        W = torch.empty(B.shape[1], m, dtype=B.dtype, device=B.device).t()  # column-major copy
        W.copy_(B)
        lmul_(self.Q.adjoint(), W)
        X = W[:n, :]
        F = self.factors
        p = _prefix(F.dtype)
        for c in range(X.shape[1]):
            col = X[:, c]
            _lib.call(f"bm_{p}tbsv", b"U", b"N", b"N", n, F.u, _ptr(F.data), F.lda, _ptr(col), 1, _stream(F.device))
        out = X.contiguous()
        return out[:, 0] if vec else out


class QRPackedQ:
    def __init__(self, F: BandedQR, adj: bool):
        self.F, self.adj = F, adj

    def adjoint(self) -> "QRPackedQ":
        return QRPackedQ(self.F, not self.adj)

    T = property(adjoint)

    def __matmul__(self, B: torch.Tensor) -> torch.Tensor:
        W = B.clone() if B.dim() == 1 else torch.empty(B.shape[1], B.shape[0], dtype=B.dtype, device=B.device).t()
        if B.dim() == 2:
            W.copy_(B)
        return lmul_(self, W)


def lmul_(Q: QRPackedQ, B: torch.Tensor) -> torch.Tensor:
    """lmul!(Q, B) / lmul!(Q', B): B (m or m x nrhs, column-major) overwritten."""
    F = Q.F.factors
    m, n = F.shape
    if B.shape[0] != m:
        raise DimensionMismatch(f"matrix A has dimensions ({m},{n}) but B has dimensions {tuple(B.shape)}")
    nrhs = 1 if B.dim() == 1 else B.shape[1]
    if B.dim() == 2 and not (B.stride(0) == 1 and B.stride(1) >= max(1, m)):
        raise ValueError("B must be column-major")
    ldb = m if B.dim() == 1 else B.stride(1)
    _lib.call(f"bm_{_prefix(F.dtype)}gbqr_lmul", b"T" if Q.adj else b"N", m, n, F.l, F.u, _ptr(F.data), F.lda,
              _ptr(Q.F.tau), Q.F.tau.numel(), nrhs, _ptr(B), max(1, ldb), _stream(F.device))
    return B


def qr(A: BandedMatrix) -> BandedQR:
    """qr(A): widen to (l, l+u) and factor (src/banded/bandedqr.jl:1-2, :30-35)."""
    _require_cuda(A.data)
    m, n = A.shape
    l, u = max(A.l, 0), max(A.u, 0)
    if (l, u) != (A.l, A.u):
        A = A.rewiden((l, u)) if A.data.shape[0] > 0 else BandedMatrix.zeros((m, n), (l, u), A.dtype, A.device)
    d = band_storage(2 * l + u + 1, n, A.dtype, A.device)
    if n:
        d[:l, :] = 0
        d[l:, :] = A.data
    F = BandedMatrix(d, m, l, l + u)
    tau = torch.zeros(min(m, n), dtype=A.dtype, device=A.device)
    if m and n:
        _lib.call(f"bm_{_prefix(A.dtype)}gbqrf", m, n, l, l + u, _ptr(d), F.lda, _ptr(tau), _stream(A.device))
    return BandedQR(F, tau)
