"""Work division across GPUs (one process per GPU), where the path shards.

* Batched solves shard by system, with no exchange: ``batch_shards`` assigns the
  systems to ranks longest-first onto the least-loaded rank (cost
  n*kl*(kl+ku) + nrhs*n*(2kl+ku), as the batch's own work queue).
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
    are shorter than the bandwidth)."""
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
            buf = torch.empty(recv_hi - recv_lo, dtype=x_local.dtype, device=x_local.device)
            parts[k] = (recv_lo, buf)
            ops.append(dist.P2POp(dist.irecv, buf, k, group))
    if ops:
        for req in dist.batch_isend_irecv(ops):
            req.wait()
    out = torch.empty(c1 - c0, dtype=x_local.dtype, device=x_local.device)
    for k, p in enumerate(parts):
        if p is None:
            continue
        if k == rank:
            out[r0 - c0: r1 - c0] = x_local
        else:
            lo, buf = p
            out[lo - c0: lo - c0 + buf.numel()] = buf
    return out


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
