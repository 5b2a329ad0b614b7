"""Work division across GPUs (one process per GPU), where the path shards.

* Batched solves shard by system, with no exchange: ``batch_shards`` assigns the
  systems to ranks longest-first onto the least-loaded rank (cost
  n*kl*(kl+ku) + nrhs*n*(2kl+ku), as the batch's own work queue).
* gbmm shards by column blocks of C (``gbmm_cols``): C's columns [j0, j1) need B's
  columns [j0, j1) and A's columns [j0 - Bu, j1 + Bl) -- a halo of A's storage
  columns from the neighbouring ranks, then one product on blocks that are bands
  themselves (shifted bandwidths over the same storage rows).
* gbmv shards by row blocks.  Rows [r0, r1) of an (l, u) band need columns
  [max(0, r0 - l), min(n, r1 + u)); that block is itself a band over the same storage
  columns, with bandwidths (l - d, u + d), d = r0 - c0 (``row_block``).  With x
  distributed in the same row blocks, each rank needs a halo of l entries of x from
  the rank before it and u entries from the rank after it: one point-to-point
  exchange (``exchange_halo``), then independent compute.  Each output row keeps its
  accumulation order, so the sharded result equals the unsharded one bit for bit.
* A single LU or QR does not shard without changing the pivot order: replicas only.
"""
from __future__ import annotations

import numpy as np
import torch


def row_ranges(m: int, world: int) -> list[tuple[int, int]]:
    """Contiguous, balanced row blocks [r0, r1) for ranks 0..world-1."""
    base, extra = divmod(m, world)
    out, r = [], 0
    for k in range(world):
        h = base + (1 if k < extra else 0)
        out.append((r, r + h))
        r += h
    return out


def row_block(m: int, n: int, l: int, u: int, r0: int, r1: int) -> dict:
    """The band block holding rows [r0, r1): its column range [c0, c1) and bandwidths.

    The block's storage is columns c0..c1-1 of the full band storage (same l+u+1 rows),
    read as an (r1-r0) x (c1-c0) band with bandwidths (l - d, u + d), d = r0 - c0."""
    c0 = max(0, r0 - l)
    c1 = min(n, r1 + u)
    d = r0 - c0
    return {"c0": c0, "c1": c1, "m": r1 - r0, "n": c1 - c0, "l": l - d, "u": u + d}


def exchange_halo(x_local: torch.Tensor, r0: int, r1: int, n: int, l: int, u: int, world: int, rank: int,
                  group=None) -> torch.Tensor:
    """x[c0:c1] for this rank's rows, from x distributed in the row blocks of
    ``row_ranges``: the last entries of lower ranks and the first entries of higher
    ranks, by point-to-point sends (the halo may span several neighbours when blocks
    are shorter than the bandwidth).  x may carry trailing dimensions (a block of
    storage columns, one per leading index)."""
    import torch.distributed as dist

    ranges = row_ranges(n, world)
    c0, c1 = max(0, r0 - l), min(n, r1 + u)
    parts = [None] * world
    parts[rank] = x_local
    ops = []
    for k, (a, b) in enumerate(ranges):
        if k == rank:
            continue
        # what rank k needs from me, and what I need from rank k
        ka, kb = ranges[k]
        kc0, kc1 = max(0, ka - l), min(n, kb + u)
        send_lo, send_hi = max(r0, kc0), min(r1, kc1)
        if send_hi > send_lo:
            ops.append(dist.P2POp(dist.isend, x_local[send_lo - r0: send_hi - r0].contiguous(), k, group))
        recv_lo, recv_hi = max(a, c0), min(b, c1)
        if recv_hi > recv_lo:
            buf = torch.empty((recv_hi - recv_lo,) + tuple(x_local.shape[1:]), dtype=x_local.dtype,
                              device=x_local.device)
            parts[k] = (recv_lo, buf)
            ops.append(dist.P2POp(dist.irecv, buf, k, group))
    if ops:
        for req in dist.batch_isend_irecv(ops):
            req.wait()
    out = torch.empty((c1 - c0,) + tuple(x_local.shape[1:]), dtype=x_local.dtype, device=x_local.device)
    for k, p in enumerate(parts):
        if p is None:
            continue
        if k == rank:
            out[r0 - c0: r1 - c0] = x_local
        else:
            lo, buf = p
            out[lo - c0: lo - c0 + buf.shape[0]] = buf
    return out


def gbmv_rows(data_block: torch.Tensor, n: int, l: int, u: int, x_local: torch.Tensor, world: int, rank: int,
              group=None, alpha: float = 1.0, out: torch.Tensor | None = None) -> torch.Tensor:
    """This rank's rows [r0, r1) (``row_ranges(n, world)[rank]``) of y = alpha A x for a
    square n x n (l, u) band, with x distributed in the same row blocks.

    ``data_block`` is the rank's slice of the band storage: columns [c0, c1) of
    ``row_block`` (all l+u+1 storage rows, column-major, on this rank's GPU).  The
    x-halo arrives by ``exchange_halo`` (x_local on the device for NCCL, on the host for
    gloo: it is moved to the band's device afterwards); the rows are then one call of
    the library's gbmv on the block read as an (r1-r0) x (c1-c0) band with bandwidths
    (l - d, u + d), d = r0 - c0 -- no further exchange.  Each output row keeps the
    unsharded accumulation order, so the gathered result equals A*x bit for bit."""
    from .banded import BandedMatrix, gbmv

    r0, r1 = row_ranges(n, world)[rank]
    blk = row_block(n, n, l, u, r0, r1)
    if data_block.shape != (l + u + 1, blk["n"]):
        raise ValueError(f"data_block must be the {l + u + 1} x {blk['n']} storage columns [{blk['c0']}, {blk['c1']})")
    if x_local.shape != (r1 - r0,):
        raise ValueError(f"x_local must hold the {r1 - r0} entries of rows [{r0}, {r1})")
    halo = exchange_halo(x_local, r0, r1, n, l, u, world, rank, group).to(data_block.device)
    y = out if out is not None else torch.empty(r1 - r0, dtype=data_block.dtype, device=data_block.device)
    if blk["m"] == 0:
        return y
    gbmv("N", alpha, BandedMatrix(data_block, blk["m"], blk["l"], blk["u"]), halo, 0.0, y)
    return y


def col_block(n: int, Al: int, Au: int, Bl: int, Bu: int, j0: int, j1: int) -> dict:
    """For C = A*B (all n x n bands) restricted to C's columns [j0, j1): A's columns
    [v0, v1) and rows [i0, i1) that enter, and the bandwidths of the three blocks.
    A block keeps its matrix's storage rows: A's columns [v0, v1) read as an
    (i1-i0) x (v1-v0) band (Al + e, Au - e), e = v0 - i0; B's columns [j0, j1) as a
    (v1-v0) x (j1-j0) band (Bl + d, Bu - d), d = j0 - v0; C's columns [j0, j1) as an
    (i1-i0) x (j1-j0) band (Cl + d + e, Cu - d - e)."""
    d = min(Bu, j0)
    v0, v1 = j0 - d, min(n, j1 + Bl)
    e = min(Au, v0)
    i0, i1 = v0 - e, min(n, v1 + Al)
    return {"v0": v0, "v1": v1, "i0": i0, "i1": i1, "d": d, "e": e}


def gbmm_cols(A_local: torch.Tensor, B_local: torch.Tensor, C_local: torch.Tensor, n: int,
              Al: int, Au: int, Bl: int, Bu: int, Cl: int, Cu: int, world: int, rank: int, group=None,
              alpha: float = 1.0, beta: float = 0.0) -> torch.Tensor:
    """This rank's columns [j0, j1) (``row_ranges(n, world)[rank]``) of C = alpha A B +
    beta C for square n x n bands, every matrix distributed by the same column blocks:
    A_local, B_local, C_local are the rank's storage columns (all bands, column-major,
    on its GPU).  The halo of A's storage columns arrives by ``exchange_halo`` (through
    host memory under gloo), then one library product on the blocks of ``col_block``.
    Each entry of C keeps the unsharded accumulation order, so the gathered result
    equals A*B bit for bit.  Returns C_local."""
    from .banded import BandedMatrix
    from .gbmm import gbmm

    j0, j1 = row_ranges(n, world)[rank]
    if B_local.shape[1] != j1 - j0 or C_local.shape[1] != j1 - j0 or A_local.shape[1] != j1 - j0:
        raise ValueError(f"the local blocks must hold the {j1 - j0} storage columns [{j0}, {j1})")
    blk = col_block(n, Al, Au, Bl, Bu, j0, j1)
    # A's storage columns [v0, v1): exchanged as rows of the transposed slab (on the host
    # for gloo, whose transport takes host memory; on the device for NCCL)
    import torch.distributed as dist

    slab = A_local.t().contiguous()
    if dist.get_backend(group) == "gloo":
        slab = slab.cpu()
    halo = exchange_halo(slab, j0, j1, n, Bu, Bl, world, rank, group)
    Ah = halo.to(A_local.device).t()  # column-major (rows, v1 - v0)
    if j1 == j0:
        return C_local
    d, e = blk["d"], blk["e"]
    m_blk = blk["i1"] - blk["i0"]
    A_blk = BandedMatrix(Ah, m_blk, Al + e, Au - e)
    B_blk = BandedMatrix(B_local, blk["v1"] - blk["v0"], Bl + d, Bu - d)
    C_blk = BandedMatrix(C_local, m_blk, Cl + d + e, Cu - d - e)
    gbmm(alpha, A_blk, B_blk, beta, C_blk)
    return C_local


def batch_shards(n, kl, ku, nrhs, world: int) -> list[np.ndarray]:
    """System indices per rank: longest first onto the least-loaded rank."""
    n, kl, ku, nrhs = (np.asarray(v, dtype=np.int64) for v in (n, kl, ku, nrhs))
    cost = n * (2 * kl * (kl + ku) + kl) + nrhs * 2 * n * (2 * kl + ku + 1)
    load = np.zeros(world)
    out = [[] for _ in range(world)]
    for s in np.argsort(-cost, kind="stable"):
        k = int(np.argmin(load))
        out[k].append(int(s))
        load[k] += cost[s]
    return [np.asarray(sorted(o), dtype=np.int64) for o in out]
