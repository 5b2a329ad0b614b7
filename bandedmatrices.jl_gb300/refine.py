"""Mixed-precision refined solve of one banded system (LAPACK DSGESV's scheme on a
band): the Float64 band is rounded to Float32 and factored with partial pivoting
(bm_sgbtrf); then x = LU32 \\ b and, until the backward error
||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf) reaches ``tol``, the residual is
formed in Float64 from the original band (bm_dgbmv) and the Float32 correction
LU32 \\ r is added in Float64.  Every step runs on the device through the library.

No counterpart in the reference; it replaces lu! + ldiv!
(src/banded/BandedLU.jl:90-103, src/banded/linalg.jl:24-30) for callers that accept
a backward-error target, and is the single-system form of bm_dsgbsv_batched.
"""
from __future__ import annotations

import torch

from .banded import BandedMatrix, band_storage
from .linalg import mul_
from .lu import lu


def solve_refined(A: BandedMatrix, b: torch.Tensor, tol: float = 1e-10, maxit: int = 50):
    """x with ||b - A x||_inf <= tol (||A||_inf ||x||_inf + ||b||_inf), A square Float64.

    Returns (x, stats) with stats = {"iters": corrections taken, "berr": final backward
    error, "info": the Float32 factorization's info}; x is all NaN-free only when the
    Float32 factorization succeeded (info == 0)."""
    if A.dtype != torch.float64 or b.dtype != torch.float64:
        raise TypeError("solve_refined refines to Float64: A and b must be Float64")
    n = A.shape[0]
    d32 = band_storage(A.data.shape[0], n, torch.float32, A.device)
    d32.copy_(A.data)
    F = lu(BandedMatrix(d32, A.m, A.l, A.u))
    cols = [b] if b.dim() == 1 else [b[:, c] for c in range(b.shape[1])]
    absA = BandedMatrix(A.data.abs(), A.m, A.l, A.u)
    ones = torch.ones(n, dtype=torch.float64, device=A.device)
    rows = torch.empty(n, dtype=torch.float64, device=A.device)
    mul_(rows, absA, ones)
    anorm = float(rows.max()) if n else 0.0
    xs, its, berr = [], 0, 0.0
    for bc in cols:
        bc = bc.contiguous()
        x = F.solve(bc.float()).double()
        bnorm = float(bc.abs().max()) if n else 0.0
        r = torch.empty_like(bc)
        it = 0
        while True:
            r.copy_(bc)
            mul_(r, A, x, -1.0, 1.0)  # r = b - A x in Float64
            den = anorm * float(x.abs().max()) + bnorm
            be = float(r.abs().max()) / den if den > 0 else float(r.abs().max())
            if not be > tol or it >= maxit:
                break
            x += F.solve(r.float()).double()
            it += 1
        xs.append(x)
        its, berr = max(its, it), max(berr, be)
    x = xs[0] if b.dim() == 1 else torch.stack(xs, dim=1)
    return x, {"iters": its, "berr": berr, "info": F.info}
