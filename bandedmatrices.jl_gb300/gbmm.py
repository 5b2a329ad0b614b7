"""Banded x banded products: mul!(C, A, B, alpha, beta) and A*B.

Host-side dispatch of gbmm! (src/banded/gbmm.jl:207-292): negative bandwidths are
removed with views, a C narrower than the product is accepted only when the
bands it lacks are exactly zero (checked on the device), and the product itself
runs in bm_dgbmm / bm_sgbmm.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .banded import BandError, BandedMatrix, DimensionMismatch, _prefix, _ptr, _require_cuda, _scalar, _stream


def _bnds(m: int, n: int) -> tuple[int, int]:
    """_bnds (src/generic/broadcast.jl:895-897): the widest bandwidths an m x n matrix has."""
    return (m - 1, n - 1)


def prodbandwidths(*As: BandedMatrix) -> tuple[int, int]:
    """prodbandwidths (src/generic/utils.jl:19-21): the bandwidths of the product A1*A2*...,
    the sums of the factors' bandwidths; (0, 0) for no factor."""
    return (sum(A.l for A in As), sum(A.u for A in As))


def _scale_band_rows(C: BandedMatrix, r0: int, r1: int, beta: float) -> None:
    """beta-scale (zero if beta == 0) the in-band entries of rows r0:r1 of C."""
    if r1 <= r0 or C.data.numel() == 0:
        return
    j = torch.arange(C.n, device=C.device)
    for r in range(C.data.shape[0]):
        k = j + r - C.u
        ok = (k >= r0) & (k < r1)
        if bool(ok.any()):
            C.data[r, ok] = 0.0 if beta == 0 else C.data[r, ok] * beta


def _scale_band_cols(C: BandedMatrix, c0: int, c1: int, beta: float) -> None:
    if c1 <= c0 or C.data.numel() == 0:
        return
    if beta == 0:
        C.data[:, c0:c1] = 0.0
    else:
        C.data[:, c0:c1] *= beta


def _row_view(M: BandedMatrix, r: int) -> BandedMatrix:
    """view(M, 1+r:end, :): same storage, bandwidths (l-r, u+r)."""
    return BandedMatrix(M.data, M.m - r, M.l - r, M.u + r)


def _col_view(M: BandedMatrix, c: int) -> BandedMatrix:
    """view(M, :, 1+c:end): storage columns shifted, bandwidths (l+c, u-c)."""
    return BandedMatrix(M.data[:, c:], M.m, M.l + c, M.u - c)


def nonzero_bands(M: BandedMatrix) -> list[bool]:
    """For each storage row (band) of M: does it hold a nonzero in-matrix entry?  (device reduction)"""
    rows = M.data.shape[0]
    flags = torch.zeros(max(rows, 1), dtype=torch.int32, device=M.device)
    if rows and M.n:
        _lib.call(f"bm_{_prefix(M.dtype)}gb_nonzero_bands", M.m, M.n, M.l, M.u, _ptr(M.data), M.lda, _ptr(flags),
                  _stream(M.device))
    return [bool(v) for v in flags[:rows].tolist()]


def _num_zeroband_u(M: BandedMatrix) -> int:
    """_num_zeroband_u (gbmm.jl:191-197): leading all-zero bands from the top."""
    f = nonzero_bands(M)
    for b, nz in enumerate(f):
        if nz:
            return b
    return len(f)


def _num_zeroband_l(M: BandedMatrix) -> int:
    f = nonzero_bands(M)
    for b, nz in enumerate(reversed(f)):
        if nz:
            return b
    return len(f)


def gbmm(alpha: float, A: BandedMatrix, B: BandedMatrix, beta: float, C: BandedMatrix) -> BandedMatrix:
    """gbmm!('N','N', alpha, A, B, beta, C): C <- alpha*A*B + beta*C."""
    _require_cuda(A.data, B.data, C.data)
    n, nu = A.shape
    if B.m != nu or C.shape != (n, B.n):
        raise DimensionMismatch(f"A is {A.shape}, B is {B.shape}, C is {C.shape}")
    if not (A.dtype == B.dtype == C.dtype):
        raise TypeError("gbmm: element types must agree")
    m = B.n
    if n == 0 or m == 0:
        return C
    Al, Au, Bl, Bu = A.l, A.u, B.l, B.u
    if -Al > Au or -Bl > Bu:
        # A or B has no bands: the reference fills C with zeros (gbmm.jl:231-233)
        C.data.zero_()
        return C
    if Al < 0:
        c = -Al
        if c >= nu:
            _scale_band_rows(C, 0, n, beta)
            return C
        return gbmm(alpha, _col_view(A, c), _row_view(B, c), beta, C)
    if Au < 0:
        r = -Au
        _scale_band_rows(C, 0, min(r, n), beta)
        if r >= n:
            return C
        gbmm(alpha, _row_view(A, r), B, beta, _row_view(C, r))
        return C
    if Bl < 0:
        c = -Bl
        _scale_band_cols(C, 0, min(c, m), beta)
        if c >= m:
            return C
        gbmm(alpha, A, _col_view(B, c), beta, _col_view(C, c))
        return C
    if Bu < 0:
        r = -Bu
        if r >= nu:
            _scale_band_rows(C, 0, n, beta)
            return C
        return gbmm(alpha, _col_view(A, r), _row_view(B, r), beta, C)

    Cl_need = min(Al + Bl, n - 1)
    Cu_need = min(Au + Bu, m - 1)
    if C.u < Cu_need:
        Au_r, Bu_r = _num_zeroband_u(A), _num_zeroband_u(B)
        if C.u < Cu_need - Au_r - Bu_r:
            raise BandError(f"C has upper bandwidth {C.u} < {Cu_need - Au_r - Bu_r}")
        if Au - Au_r < -Al or Bu - Bu_r < -Bl:
            _scale_band_rows(C, 0, n, beta)
            return C
        At = BandedMatrix(A.data[Au_r:, :], A.m, Al, Au - Au_r)
        Bt = BandedMatrix(B.data[Bu_r:, :], B.m, Bl, Bu - Bu_r)
        return gbmm(alpha, At, Bt, beta, C)
    if C.l < Cl_need:
        Al_r, Bl_r = _num_zeroband_l(A), _num_zeroband_l(B)
        if C.l < Cl_need - Al_r - Bl_r:
            raise BandError(f"C has lower bandwidth {C.l} < {Cl_need - Al_r - Bl_r}")
        if Al - Al_r < -Au or Bl - Bl_r < -Bu:
            _scale_band_rows(C, 0, n, beta)
            return C
        At = BandedMatrix(A.data[:A.data.shape[0] - Al_r, :], A.m, Al - Al_r, Au)
        Bt = BandedMatrix(B.data[:B.data.shape[0] - Bl_r, :], B.m, Bl - Bl_r, Bu)
        return gbmm(alpha, At, Bt, beta, C)

    if C.l < 0 or C.u < 0:
        # C's band lies off one side of the diagonal; compute into a widened copy
        W = BandedMatrix.zeros(C.shape, (max(C.l, 0), max(C.u, 0)), C.dtype, C.device)
        W.data[max(C.u, 0) - C.u: max(C.u, 0) - C.u + C.data.shape[0], :] = C.data
        gbmm(alpha, A, B, beta, W)
        C.data.copy_(W.data[max(C.u, 0) - C.u: max(C.u, 0) - C.u + C.data.shape[0], :])
        return C
    _lib.call(f"bm_{_prefix(A.dtype)}gbmm", n, nu, m, Al, Au, Bl, Bu, C.l, C.u, _scalar(A.dtype, alpha),
              _ptr(A.data), A.lda, _ptr(B.data), B.lda, _scalar(A.dtype, beta), _ptr(C.data), C.lda,
              _stream(A.device))
    return C


def banded_mul_(C: BandedMatrix, A: BandedMatrix, B: BandedMatrix, alpha: float = 1.0,
                beta: float = 0.0) -> BandedMatrix:
    """mul!(C, A, B, alpha, beta) for banded A, B, C (materialize!, src/generic/matmul.jl:186-189)."""
    return gbmm(alpha, A, B, beta, C)


def banded_mul(A: BandedMatrix, B: BandedMatrix) -> BandedMatrix:
    """A * B: result bandwidths min(_bnds, prodbandwidths) (src/generic/matmul.jl:1-6)."""
    if A.n != B.m:
        raise DimensionMismatch(f"A is {A.shape}, B is {B.shape}")
    n, m = A.m, B.n
    bl, bu = _bnds(n, m)
    pl, pu = prodbandwidths(A, B)
    l, u = min(bl, pl), min(bu, pu)
    C = BandedMatrix.zeros((n, m), (l, u), A.dtype, A.device)
    if l + u + 1 <= 0:
        return C
    return gbmm(1.0, A, B, 0.0, C)
