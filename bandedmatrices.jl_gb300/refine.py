"""Mixed-precision refined solve of one banded system (LAPACK DSGESV's scheme on a
band), through bm_dsgbsv: the Float64 band is factored in Float32 with partial
pivoting (for 64 <= l+u <= 256 by the tensor-core blocked LU), then x = LU32 \\ b and,
until the backward error ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf) reaches
``tol``, the residual is formed in Float64 from the original band and the Float32
correction LU32 \\ r is added in Float64.  The whole loop is enqueued in one call and
decided on the device: no host synchronisation until the caller reads the result.

No counterpart in the reference; it replaces lu! + ldiv!
(src/banded/BandedLU.jl:90-103, src/banded/linalg.jl:24-30) for callers that accept
a backward-error target, and is the single-system form of bm_dsgbsv_batched.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .banded import BandedMatrix, _ptr, _require_cuda, _stream


def solve_refined(A: BandedMatrix, b: torch.Tensor, tol: float = 1e-10, maxit: int = 30):
    """x with ||b - A x||_inf <= tol (||A||_inf ||x||_inf + ||b||_inf), A square Float64
    with bandwidths 0 <= l, u and l + u <= 256; b of length n, or n x nrhs.

    Returns (x, stats): stats = {"iters": corrections taken, "berr": final backward
    error, "info": the Float32 factorization's info} as 0-d device tensors (reading
    them synchronises); x is meaningful only when info == 0."""
    if A.dtype != torch.float64 or b.dtype != torch.float64:
        raise TypeError("solve_refined refines to Float64: A and b must be Float64")
    if A.m != A.n:
        raise ValueError("solve_refined needs a square matrix")
    if A.l < 0 or A.u < 0:
        raise ValueError("solve_refined needs non-negative bandwidths")
    _require_cuda(A.data, b)
    n, kl, ku = A.n, A.l, A.u
    B = b.reshape(n, -1) if b.dim() == 1 else b
    nrhs = B.shape[1]
    Bc = B.t().contiguous().t() if nrhs else B  # column-major, leading dim n
    dev = A.device
    X = torch.empty(nrhs, n, dtype=torch.float64, device=dev).t()
    ipiv = torch.empty(max(n, 1), dtype=torch.int64, device=dev)
    ldf = (2 * kl + ku + 1 + 3) // 4 * 4
    swork = torch.empty(ldf * n + n * nrhs + 1, dtype=torch.float32, device=dev)
    work = torch.empty(n * nrhs + 3 * nrhs + 2, dtype=torch.float64, device=dev)
    it = torch.empty(1, dtype=torch.int32, device=dev)
    berr = torch.empty(1, dtype=torch.float64, device=dev)
    info = torch.empty(1, dtype=torch.int64, device=dev)
    _lib.call("bm_dsgbsv", n, kl, ku, nrhs, _ptr(A.data), A.lda, _ptr(Bc), max(1, n), _ptr(X), max(1, n), _ptr(ipiv),
              _ptr(swork), _ptr(work), ctypes.c_double(tol), int(maxit), _ptr(it), _ptr(berr), _ptr(info),
              _stream(dev))
    x = X[:, 0] if b.dim() == 1 else X
    return x, {"iters": it[0], "berr": berr[0], "info": info[0]}
