"""Format conversion of device BandedMatrix objects: sparse(A) (a torch sparse CSC
tensor, ext/BandedMatricesSparseArraysExt.jl:7-9), bandwidths(S) of a sparse matrix
(:11-33), BandedMatrix(S) from a sparse CSC matrix, and the BandedRows copy from
row-major band data (src/banded/BandedMatrix.jl:267-284).  Every pass runs in
libbandedgpu (bm_{d,s}gb2csc, csc_bandwidths, csc2gb, gbrows2cols).
"""
from __future__ import annotations

import torch

from . import _lib
from .banded import BandedMatrix, _prefix, _ptr, _require_cuda, _stream, band_storage


def sparse(A: BandedMatrix) -> torch.Tensor:
    """sparse(A): a torch sparse CSC tensor holding every in-matrix band slot (explicit
    zeros included), with the reference's structure."""
    _require_cuda(A.data)
    m, n = A.shape
    nnz = int(_lib.load().bm_gb2csc_nnz(m, n, A.l, A.u))
    colptr = torch.empty(n + 1, dtype=torch.int64, device=A.device)
    rowval = torch.empty(max(nnz, 1), dtype=torch.int64, device=A.device)
    nzval = torch.empty(max(nnz, 1), dtype=A.dtype, device=A.device)
    _lib.call(f"bm_{_prefix(A.dtype)}gb2csc", m, n, A.l, A.u, _ptr(A.data), A.lda, _ptr(colptr), _ptr(rowval),
              _ptr(nzval), _stream(A.device))
    return torch.sparse_csc_tensor(colptr, rowval[:nnz], nzval[:nnz], (m, n))


def _csc_parts(S: torch.Tensor):
    if S.layout != torch.sparse_csc:
        S = S.to_sparse_csc()
    return S.ccol_indices().to(torch.int64).contiguous(), S.row_indices().to(torch.int64).contiguous(), \
        S.values().contiguous(), S


def sparse_bandwidths(S: torch.Tensor) -> tuple[int, int]:
    """bandwidths(S) for a sparse matrix: the extreme diagonals of its nonzero values."""
    colptr, rowval, vals, S = _csc_parts(S)
    _require_cuda(vals)
    m, n = S.shape
    lu = torch.empty(2, dtype=torch.int64, device=vals.device)
    _lib.call(f"bm_{_prefix(vals.dtype)}csc_bandwidths", m, n, _ptr(colptr), _ptr(rowval), _ptr(vals), _ptr(lu),
              _stream(vals.device))
    l, u = (int(v) for v in lu.cpu())
    return l, u


def from_sparse(S: torch.Tensor, bands=None) -> BandedMatrix:
    """BandedMatrix(S) (bandwidths(S) by default) or BandedMatrix(S, (l, u)); raises
    ValueError when a nonzero of S lies outside the requested band."""
    colptr, rowval, vals, S = _csc_parts(S)
    _require_cuda(vals)
    m, n = S.shape
    l, u = bands if bands is not None else sparse_bandwidths(S)
    A = BandedMatrix(band_storage(max(0, l + u + 1), n, vals.dtype, vals.device), m, l, u)
    dropped = torch.empty(1, dtype=torch.int64, device=vals.device)
    _lib.call(f"bm_{_prefix(vals.dtype)}csc2gb", m, n, _ptr(colptr), _ptr(rowval), _ptr(vals), l, u, _ptr(A.data),
              A.lda, _ptr(dropped), _stream(vals.device))
    if bands is not None and int(dropped.item()) != 0:
        raise ValueError(f"{int(dropped.item())} nonzero entries lie outside the bands ({l}, {u})")
    return A


def from_rows(R: torch.Tensor, m: int, n: int, l: int, u: int) -> BandedMatrix:
    """BandedMatrix from row-major band data: R is m x (l+u+1) with R[i, c - i + l] =
    A(i, c) (the BandedRows layout); returns column-major band storage."""
    _require_cuda(R)
    if R.shape != (m, l + u + 1):
        raise ValueError(f"R must be {m} x {l + u + 1}")
    Rc = R.t().contiguous().t()  # column-major, leading dim m
    A = BandedMatrix(band_storage(l + u + 1, n, R.dtype, R.device, fill=0.0), m, l, u)
    _lib.call(f"bm_{_prefix(R.dtype)}gbrows2cols", m, n, l, u, _ptr(Rc), max(1, m), _ptr(A.data), A.lda,
              _stream(R.device))
    return A
