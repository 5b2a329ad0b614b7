"""Differentiable banded solve: x = A \\ b with a hand-written adjoint.

``banded_solve(data, b, l, u)`` is a torch.autograd.Function: the forward pass factors
A (bm_{d,s}gbtrf) and solves (bm_{d,s}gbtrs 'N'); the backward pass calls
bm_{d,s}gbsv_adjoint, which reuses the stored factors and pivots in a transposed
solve, dL/db = A^{-T} dL/dx, and forms dL/dA = -(A^{-T} dL/dx) x^T restricted to the
band (the gradient with respect to ``data``, in the same band layout).  With
``recompute_x=True`` the forward pass keeps b instead of x and the backward pass
recomputes x from the factors, trading one more solve for the memory of x.
This is the rrule the Julia binding attaches to ``\\`` (ChainRules), built on
ldiv!(transpose(F), B) (src/banded/linalg.jl:41-47).
"""
from __future__ import annotations

import torch

from . import _lib
from .banded import BandedMatrix, _prefix, _ptr, _stream, band_storage
from .lu import lu


class BandedSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, data: torch.Tensor, b: torch.Tensor, l: int, u: int, recompute_x: bool):
        n = data.shape[1]
        d = band_storage(l + u + 1, n, data.dtype, data.device)
        d.copy_(data.detach())  # any memory layout in, LAPACK band storage for the library
        A = BandedMatrix(d, n, l, u)
        F = lu(A)
        x = F.solve(b.detach())
        ctx.l, ctx.u, ctx.recompute = l, u, recompute_x
        ctx.F = F
        ctx.vec = b.dim() == 1
        ctx.save_for_backward(b.detach() if recompute_x else x)
        return x

    @staticmethod
    def backward(ctx, gx: torch.Tensor):
        (saved,) = ctx.saved_tensors
        F = ctx.F
        n = F.shape[0]
        l, u = ctx.l, ctx.u
        nrhs = 1 if ctx.vec else gx.shape[1]

        def colmajor(t):
            if ctx.vec:
                return t.contiguous()
            out = torch.empty(t.shape[1], t.shape[0], dtype=t.dtype, device=t.device).t()
            out.copy_(t)
            return out

        Wc = colmajor(gx)
        Sc = colmajor(saved)
        gB = torch.empty_like(Wc)
        gband = torch.empty(n, l + u + 1, dtype=gx.dtype, device=gx.device).t()  # (l+u+1) x n column-major
        Xwork = torch.empty_like(Wc) if ctx.recompute else None
        p = _prefix(gx.dtype)
        null = None
        _lib.call(f"bm_{p}gbsv_adjoint", n, F.l, F.u, nrhs, _ptr(F.factors.data), F.factors.lda, _ptr(F.ipiv),
                  null if ctx.recompute else _ptr(Sc), _ptr(Sc) if ctx.recompute else null, _ptr(Wc), _ptr(gB),
                  _ptr(gband), l + u + 1, _ptr(Xwork) if ctx.recompute else null, _stream(gx.device))
        grad_b = gB if ctx.vec else gB.contiguous()
        return gband, grad_b, None, None, None


def banded_solve(data: torch.Tensor, b: torch.Tensor, l: int, u: int, recompute_x: bool = False) -> torch.Tensor:
    """x = A \\ b for the square band A with storage ``data`` ((l+u+1) x n) and bandwidths (l, u),
    differentiable with respect to ``data`` (band entries) and ``b``."""
    return BandedSolve.apply(data, b, l, u, recompute_x)
