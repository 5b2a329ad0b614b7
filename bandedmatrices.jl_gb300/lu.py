"""BandedLU on the device: lu, ldiv!, \\ and the transposed solve.

Mirrors src/banded/BandedLU.jl and src/banded/linalg.jl: ``lu(A)`` re-widens A to
bandwidths (l, l+u) (_lu, BandedLU.jl:108-111) and factors it with xGBTRF
(lu!, :90-103); ``ldiv_(F, B)`` runs xGBTRS 'N' (linalg.jl:24-30) and
``ldiv_(transpose(F), B)`` xGBTRS 'T' (:41-47).  Pivots are 1-based int64 on the
device, as BandedLU.ipiv.  Unlike the reference, which stores info = 0
unconditionally (BandedLU.jl:102), ``info`` holds LAPACK's value, so
``issuccess`` reports a zero pivot.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .banded import (BandedMatrix, DimensionMismatch, _prefix, _ptr, _require_cuda, _stream, band_storage)


class BandedLU:
    """Factorization object: ``factors`` (BandedMatrix, bandwidths (l, l+u)), ``ipiv``, ``info``."""

    def __init__(self, factors: BandedMatrix, ipiv: torch.Tensor, info: torch.Tensor, l: int, u: int):
        self.factors, self.ipiv, self.info_t, self.l, self.u = factors, ipiv, info, l, u

    # size (BandedLU.jl:49-50)
    @property
    def shape(self):
        return self.factors.shape

    def size(self, k=None):
        if k is None:
            return self.shape
        if k < 1:
            raise IndexError("dimension out of range")
        return self.shape[k - 1] if k <= 2 else 1

    @property
    def info(self) -> int:
        return int(self.info_t.item())

    def issuccess(self) -> bool:
        return self.info == 0

    def transpose(self) -> "TransposedBandedLU":
        return TransposedBandedLU(self)

    T = property(transpose)

    def adjoint(self) -> "TransposedBandedLU":
        return TransposedBandedLU(self)  # real element types: adjoint == transpose (linalg.jl:55-56)

    def solve(self, B: torch.Tensor) -> torch.Tensor:
        """F \\ B (copies B)."""
        return ldiv_(self, B.clone())

    def inv_norm1_estimate(self, maxit: int = 5) -> float:
        """Estimate of ||A^{-1}||_1 from the factors, the quantity LAPACK's xGBCON
        estimates with xLACN2: Hager's method with Higham's refinements (sign vector,
        stop when the gradient does not grow), two triangular-solve pairs per iteration
        on the device."""
        n = self.shape[0]
        dev, dt = self.factors.data.device, self.factors.data.dtype
        x = torch.full((n,), 1.0 / n, dtype=dt, device=dev)
        est, last_j = 0.0, -1
        for it in range(maxit):
            y = self.solve(x)
            new = float(y.abs().sum())
            if it > 0 and new <= est:
                break
            est = new
            z = TransposedBandedLU(self).solve(torch.where(y >= 0, 1.0, -1.0).to(dt))
            j = int(z.abs().argmax())
            if it > 0 and (j == last_j or float(z.abs().max()) <= float((z * x).sum())):
                break
            last_j = j
            x = torch.zeros(n, dtype=dt, device=dev)
            x[j] = 1.0
        # Higham's alternative estimate (the alternating-sign vector)
        alt = torch.arange(n, dtype=dt, device=dev)
        alt = (1.0 + alt / max(n - 1, 1)) * torch.where(alt.remainder(2) == 0, 1.0, -1.0).to(dt)
        est2 = 2.0 * float(self.solve(alt).abs().sum()) / (3.0 * n)
        return max(est, est2)

    # -- L, U, p, P (BandedLU.jl:114-130): dense host-side views for inspection/tests
    @property
    def p(self) -> np.ndarray:
        m = self.shape[0]
        perm = np.arange(m)
        ip = self.ipiv.cpu().numpy()
        for i, v in enumerate(ip):
            j = v - 1
            perm[i], perm[j] = perm[j], perm[i]
        return perm + 1

    @property
    def U(self) -> np.ndarray:
        m, n = self.shape
        D = self.factors.to_dense().cpu().numpy()
        return np.triu(D[: min(m, n), :])

    @property
    def L(self) -> np.ndarray:
        m, n = self.shape
        kv = self.factors.u
        data = self.factors.data.cpu().numpy()
        ip = self.ipiv.cpu().numpy() - 1
        L = np.eye(m, min(m, n), dtype=data.dtype)
        cols = []
        for j in range(min(m, n)):
            p = ip[j]
            for prev in cols:
                prev[[j, p]] = prev[[p, j]]
            col = np.zeros(m, dtype=data.dtype)
            for i in range(j + 1, min(m, j + self.l + 1)):
                col[i] = data[kv + i - j, j]
            cols.append(col)
        for j, col in enumerate(cols):
            L[:, j] += col
        return L


class TransposedBandedLU:
    def __init__(self, F: BandedLU):
        self.parent = F

    def solve(self, B: torch.Tensor) -> torch.Tensor:
        return ldiv_(self, B.clone())


def transpose(F: BandedLU) -> TransposedBandedLU:
    return F.transpose()


def lu(A: BandedMatrix) -> BandedLU:
    """lu(A): copy into (l, l+u) gbtrf storage and factor (BandedLU.jl:108-111, :90-103)."""
    _require_cuda(A.data)
    m, n = A.shape
    l, u = max(A.l, 0), max(A.u, 0)
    if (l, u) != (A.l, A.u) and A.data.shape[0] > 0:
        A = A.rewiden((l, u))
    elif A.data.shape[0] == 0:
        A = BandedMatrix.zeros((m, n), (l, u), A.dtype, A.device)
    # factors: bandwidths (l, l+u) -> 2l+u+1 storage rows, top l rows zero
    d = band_storage(2 * l + u + 1, n, A.dtype, A.device)
    if n:
        d[:l, :] = 0
        d[l:, :] = A.data
    F = BandedMatrix(d, m, l, l + u)
    ipiv = torch.zeros(max(0, min(m, n)), dtype=torch.int64, device=A.device)
    info = torch.zeros(1, dtype=torch.int64, device=A.device)
    if m and n:
        _lib.call(f"bm_{_prefix(A.dtype)}gbtrf", m, n, l, u, _ptr(d), F.lda, _ptr(ipiv), _ptr(info), _stream(A.device))
    return BandedLU(F, ipiv, info, l, u)


def lu_(F_storage: BandedMatrix) -> BandedLU:
    """lu!(A) on a BandedMatrix that already has bandwidths (l, l+u): factors in place."""
    m, n = F_storage.shape
    l = F_storage.l
    u = F_storage.u - l
    ipiv = torch.zeros(max(0, min(m, n)), dtype=torch.int64, device=F_storage.device)
    info = torch.zeros(1, dtype=torch.int64, device=F_storage.device)
    if m and n:
        _lib.call(f"bm_{_prefix(F_storage.dtype)}gbtrf", m, n, l, u, _ptr(F_storage.data), F_storage.lda, _ptr(ipiv),
                  _ptr(info), _stream(F_storage.device))
    return BandedLU(F_storage, ipiv, info, l, u)


def _as_colmajor(B: torch.Tensor) -> tuple[torch.Tensor, bool]:
    """Column-major (n, nrhs) working copy of B if B is not already one."""
    if B.dim() == 1:
        return B, False
    if B.stride(0) == 1 and B.stride(1) >= max(1, B.shape[0]):
        return B, False
    W = torch.empty(B.shape[1], B.shape[0], dtype=B.dtype, device=B.device).t()
    W.copy_(B)
    return W, True


def ldiv_(F, B: torch.Tensor) -> torch.Tensor:
    """ldiv!(F, B) / ldiv!(transpose(F), B): B is overwritten with the solution."""
    trans = isinstance(F, TransposedBandedLU)
    G = F.parent if trans else F
    _require_cuda(B)
    m, n = G.shape
    if m != n:
        raise DimensionMismatch(f"matrix is not square: dimensions are ({m}, {n})")
    if B.shape[0] != n:
        raise DimensionMismatch(f"B has leading dimension {B.shape[0]}, but needs {n}")
    if B.dtype != G.factors.dtype:
        raise TypeError("element types of the factors and B must agree")
    if n == 0 or B.numel() == 0:
        return B
    W, copied = _as_colmajor(B)
    nrhs = 1 if W.dim() == 1 else W.shape[1]
    ldb = n if W.dim() == 1 else W.stride(1)
    if W.dim() == 1 and W.stride(0) != 1:
        W = W.contiguous()
        copied = True
    _lib.call(f"bm_{_prefix(W.dtype)}gbtrs", b"T" if trans else b"N", n, G.l, G.u, nrhs, _ptr(G.factors.data),
              G.factors.lda, _ptr(G.ipiv), _ptr(W), ldb, _stream(W.device))
    if copied:
        B.copy_(W)
    return B
