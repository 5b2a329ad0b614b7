"""The multi-GPU splits through the library (GPU), as two gloo ranks on one GPU:
* gbmv by row blocks (``shard.gbmv_rows``): each rank holds only its slice of the band
  storage and its rows of x, exchanges the x-halo on the host and computes its rows
  with the library's gbmv;
* gbmm by column blocks (``shard.gbmm_cols``): each rank holds its storage columns of
  A, B and C, exchanges the halo of A's columns and computes its columns of C with
  the library's product.
The gathered results equal the unsharded library calls and the oracle bit for bit.
The ranks' kernels never wait on one another: the only exchanges are host-side."""
import os
import socket
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WORLD = 2
CASES = [(5000, 7, 4, "f64"), (37, 30, 2, "f64"), (4096, 0, 0, "f32"), (900, 3, 60, "f32"), (100003, 32, 32, "f64")]
MM_CASES = [(500, 3, 4, 2, 5, "f64"), (37, 10, 2, 1, 12, "f64"), (3000, 16, 16, 16, 16, "f32"),
            (2001, 0, 3, 4, 0, "f64")]


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
    for case, (n, Al, Au, Bl, Bu, dt) in enumerate(MM_CASES):
        nt = np.float64 if dt == "f64" else np.float32
        tdt = torch.float64 if dt == "f64" else torch.float32
        rng = np.random.default_rng(300 + case)
        Ad = rng.standard_normal((Al + Au + 1, n)).astype(nt)
        Bd = rng.standard_normal((Bl + Bu + 1, n)).astype(nt)
        Cl, Cu = Al + Bl, Au + Bu
        j0, j1 = bm.shard.row_ranges(n, WORLD)[rank]

        def slab(data, rows):
            t = bm.band_storage(rows, j1 - j0, tdt, dev)
            t.copy_(torch.from_numpy(np.ascontiguousarray(data[:, j0:j1])))
            return t

        Cl_t = bm.band_storage(Cl + Cu + 1, j1 - j0, tdt, dev)
        Cl_t.fill_(float("nan"))  # every slot of the rank's columns is written
        bm.shard.gbmm_cols(slab(Ad, Al + Au + 1), slab(Bd, Bl + Bu + 1), Cl_t, n, Al, Au, Bl, Bu, Cl, Cu, WORLD,
                           rank)
        torch.cuda.synchronize()
        parts = [None] * WORLD
        dist.all_gather_object(parts, Cl_t.cpu().numpy())
        res[f"C{case}"] = np.concatenate(parts, axis=1)
        if rank == 0:
            A = bm.BandedMatrix(bm.band_storage(Al + Au + 1, n, tdt, dev), n, Al, Au)
            A.data.copy_(torch.from_numpy(Ad))
            B = bm.BandedMatrix(bm.band_storage(Bl + Bu + 1, n, tdt, dev), n, Bl, Bu)
            B.data.copy_(torch.from_numpy(Bd))
            res[f"Cfull{case}"] = bm.banded_mul(A, B).data.cpu().numpy()
            res[f"Ad{case}"], res[f"Bd{case}"] = Ad, Bd
    dist.barrier()
    dist.destroy_process_group()
    np.savez(os.path.join(outdir, f"rank{rank}.npz"), **res)


def test_two_rank_gbmv_rows_and_gbmm_cols_through_the_library(tmp_path, orc):
    import torch.multiprocessing as mp

    mp.start_processes(_rank_main, args=(_free_port(), str(tmp_path)), nprocs=WORLD, start_method="spawn")
    r0 = np.load(tmp_path / "rank0.npz")
    r1 = np.load(tmp_path / "rank1.npz")
    for case, (n, l, u, dt) in enumerate(CASES):
        assert np.array_equal(r0[f"y{case}"], r1[f"y{case}"])
        assert np.array_equal(r0[f"y{case}"], r0[f"yfull{case}"]), case
        ref = orc.gbmv("N", n, n, l, u, 1.0, r0[f"data{case}"], r0[f"x{case}"])
        assert np.array_equal(r0[f"y{case}"], ref), case
    for case, (n, Al, Au, Bl, Bu, dt) in enumerate(MM_CASES):
        C = r0[f"C{case}"]
        Cl, Cu = Al + Bl, Au + Bu
        rr = np.arange(Cl + Cu + 1)[:, None] + np.arange(n)[None, :] - Cu
        mask = (rr >= 0) & (rr < n)  # the in-matrix slots of C's band storage
        assert np.array_equal(C[mask], r1[f"C{case}"][mask])
        assert not np.isnan(C[mask]).any(), case  # every in-matrix slot written
        assert np.array_equal(C[mask], r0[f"Cfull{case}"][mask]), case
        ref = orc.gbmm_percol(n, n, n, Al, Au, Bl, Bu, 1.0, r0[f"Ad{case}"], r0[f"Bd{case}"], 0.0,
                              np.zeros((Cl + Cu + 1, n), dtype=C.dtype))
        assert np.array_equal(C[mask], ref[mask]), case
