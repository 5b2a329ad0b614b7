"""The multi-GPU division of work, run as two gloo ranks on the CPU: gbmv row blocks
with the x-halo exchange (each rank computes its rows from its band block with the
oracle's gbmv; the gathered result equals the unsharded one bit for bit), gbmm column
blocks with the halo of A's storage columns (each rank's product of the blocks by the
oracle's banded product equals the unsharded one bit for bit) and the batched solves'
system assignment (a disjoint, balanced cover, identical on every rank)."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WORLD = 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _load_shard():
    import importlib.util

    spec = importlib.util.spec_from_file_location("bm_shard", os.path.join(ROOT, "bandedmatrices.jl_gb300", "shard.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _rank_main(rank, port, outdir):
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    import oracle

    shard = _load_shard()
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", world_size=WORLD, rank=rank)
    res = {}
    for case, (n, l, u) in enumerate([(500, 7, 4), (37, 30, 2), (64, 0, 0), (90, 3, 60)]):
        rng = np.random.default_rng(100 + case)
        data = np.asfortranarray(rng.standard_normal((l + u + 1, n)))
        x = rng.standard_normal(n)
        r0, r1 = shard.row_ranges(n, WORLD)[rank]
        halo = shard.exchange_halo(torch.from_numpy(x[r0:r1].copy()), r0, r1, n, l, u, WORLD, rank).numpy()
        blk = shard.row_block(n, n, l, u, r0, r1)
        assert np.array_equal(halo, x[blk["c0"]:blk["c1"]])
        y = oracle.gbmv("N", blk["m"], blk["n"], blk["l"], blk["u"], 1.0,
                        np.asfortranarray(data[:, blk["c0"]:blk["c1"]]), halo)
        parts = [None] * WORLD
        dist.all_gather_object(parts, y)
        res[f"y{case}"] = np.concatenate(parts)
        res[f"yref{case}"] = oracle.gbmv("N", n, n, l, u, 1.0, data, x)
    # gbmm by column blocks: the halo of A's storage columns, then the product of the blocks
    for case, (n, Al, Au, Bl, Bu) in enumerate([(300, 3, 4, 2, 5), (37, 10, 2, 1, 12), (200, 0, 3, 4, 0)]):
        rng = np.random.default_rng(400 + case)
        Ad = np.asfortranarray(rng.standard_normal((Al + Au + 1, n)))
        Bd = np.asfortranarray(rng.standard_normal((Bl + Bu + 1, n)))
        Cl, Cu = Al + Bl, Au + Bu
        j0, j1 = shard.row_ranges(n, WORLD)[rank]
        blk = shard.col_block(n, Al, Au, Bl, Bu, j0, j1)
        halo = shard.exchange_halo(torch.from_numpy(np.ascontiguousarray(Ad[:, j0:j1].T)), j0, j1, n, Bu, Bl, WORLD,
                                   rank).numpy().T
        assert np.array_equal(halo, Ad[:, blk["v0"]:blk["v1"]])
        d, e = blk["d"], blk["e"]
        mb = blk["i1"] - blk["i0"]
        Cb = oracle.gbmm_generic(mb, blk["v1"] - blk["v0"], j1 - j0, Al + e, Au - e, Bl + d, Bu - d, Cl + d + e,
                                 Cu - d - e, 1.0, np.asfortranarray(halo), np.asfortranarray(Bd[:, j0:j1]), 0.0,
                                 np.zeros((Cl + Cu + 1, j1 - j0)))
        parts = [None] * WORLD
        dist.all_gather_object(parts, Cb)
        res[f"C{case}"] = np.concatenate(parts, axis=1)
        res[f"Cref{case}"] = oracle.gbmm_generic(n, n, n, Al, Au, Bl, Bu, Cl, Cu, 1.0, Ad, Bd, 0.0,
                                                 np.zeros((Cl + Cu + 1, n)))
    rng = np.random.default_rng(5)
    cnt = 300
    n = np.exp(rng.uniform(np.log(64), np.log(4000), cnt)).astype(np.int64)
    kl, ku, nrhs = rng.integers(1, 40, cnt), rng.integers(1, 40, cnt), rng.integers(1, 9, cnt)
    mine = shard.batch_shards(n, kl, ku, nrhs, WORLD)[rank]
    everyone = [None] * WORLD
    dist.all_gather_object(everyone, mine.tolist())
    res["shards"] = np.array(everyone, dtype=object)
    cost = n * (2 * kl * (kl + ku) + kl) + nrhs * 2 * n * (2 * kl + ku + 1)
    res["cost"] = cost
    dist.barrier()
    dist.destroy_process_group()
    np.savez(os.path.join(outdir, f"rank{rank}.npz"), **res)


def test_two_rank_gbmv_halo_and_batched_shards(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    import oracle

    oracle.build()
    mp.start_processes(_rank_main, args=(_free_port(), str(tmp_path)), nprocs=WORLD, start_method="spawn")
    for rank in range(WORLD):
        r = np.load(tmp_path / f"rank{rank}.npz", allow_pickle=True)
        for case in range(4):
            assert np.array_equal(r[f"y{case}"], r[f"yref{case}"]), (rank, case)
        for case in range(3):
            assert np.array_equal(r[f"C{case}"], r[f"Cref{case}"]), (rank, "gbmm", case)
        shards = [np.asarray(list(s), dtype=np.int64) for s in r["shards"]]
        allidx = np.sort(np.concatenate(shards))
        assert np.array_equal(allidx, np.arange(len(r["cost"])))  # disjoint cover
        loads = [r["cost"][s].sum() for s in shards]
        assert max(loads) <= 1.05 * sum(loads) / WORLD + r["cost"].max()
