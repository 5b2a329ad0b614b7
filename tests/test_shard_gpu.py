"""The row-block split of gbmv through the library (GPU): two gloo ranks, each holding
only its slice of the band storage and its rows of x, exchange the x-halo on the host
and compute their rows with the library's gbmv on the GPU (``shard.gbmv_rows``); the
gathered result equals the unsharded bm gbmv and the oracle bit for bit.  The ranks'
kernels never wait on one another: the only exchange is the host-side halo."""
import os
import socket
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WORLD = 2
CASES = [(5000, 7, 4, "f64"), (37, 30, 2, "f64"), (4096, 0, 0, "f32"), (900, 3, 60, "f32"), (100003, 32, 32, "f64")]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, outdir):
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    import __graft_entry__ as ge

    bm = ge.package()
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", world_size=WORLD, rank=rank)
    dev = torch.device("cuda", 0)
    res = {}
    for case, (n, l, u, dt) in enumerate(CASES):
        nt = np.float64 if dt == "f64" else np.float32
        rng = np.random.default_rng(200 + case)
        data = rng.standard_normal((l + u + 1, n)).astype(nt)
        x = rng.standard_normal(n).astype(nt)
        r0, r1 = bm.shard.row_ranges(n, WORLD)[rank]
        blk = bm.shard.row_block(n, n, l, u, r0, r1)
        dblk = bm.band_storage(l + u + 1, blk["n"], torch.from_numpy(data).dtype, dev)
        dblk.copy_(torch.from_numpy(np.ascontiguousarray(data[:, blk["c0"]:blk["c1"]])))
        y = bm.shard.gbmv_rows(dblk, n, l, u, torch.from_numpy(x[r0:r1].copy()), WORLD, rank)
        torch.cuda.synchronize()
        parts = [None] * WORLD
        dist.all_gather_object(parts, y.cpu().numpy())
        res[f"y{case}"] = np.concatenate(parts)
        if rank == 0:
            A = bm.BandedMatrix(bm.band_storage(l + u + 1, n, torch.from_numpy(data).dtype, dev), n, l, u)
            A.data.copy_(torch.from_numpy(data))
            res[f"yfull{case}"] = bm.mul(A, torch.from_numpy(x).to(dev)).cpu().numpy()
            res[f"data{case}"], res[f"x{case}"] = data, x
    dist.barrier()
    dist.destroy_process_group()
    np.savez(os.path.join(outdir, f"rank{rank}.npz"), **res)


def test_two_rank_gbmv_rows_through_the_library(tmp_path, orc):
    import torch.multiprocessing as mp

    mp.start_processes(_rank_main, args=(_free_port(), str(tmp_path)), nprocs=WORLD, start_method="spawn")
    r0 = np.load(tmp_path / "rank0.npz")
    r1 = np.load(tmp_path / "rank1.npz")
    for case, (n, l, u, dt) in enumerate(CASES):
        assert np.array_equal(r0[f"y{case}"], r1[f"y{case}"])
        assert np.array_equal(r0[f"y{case}"], r0[f"yfull{case}"]), case
        ref = orc.gbmv("N", n, n, l, u, 1.0, r0[f"data{case}"], r0[f"x{case}"])
        assert np.array_equal(r0[f"y{case}"], ref), case
