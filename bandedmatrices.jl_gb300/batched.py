"""Batched banded solves: thousands of independent systems of uneven n, (kl, ku)
and right-hand-side counts in one persistent launch (bm_{d,s}gbsv_batched).

The batch owns three flat device buffers -- every system's gbtrf band storage,
right-hand sides and pivots -- plus a device descriptor table.  Systems are
handed out from a device work queue in longest-processing-time order (cost
n*kl*(kl+ku), largest first) so that the tail of the launch stays short.  The
launch performs no allocation and no host synchronisation, so a whole solve can
be captured once in a CUDA graph and replayed.

Launch schedule: "wide" systems (more than ``narrow_cols`` band columns) are solved
one at a time by a CTA of 4 or 8 warps, "narrow" ones one per warp.  ``tune()`` is
the autotuner: it times candidate schedules on the batch itself and keeps the
fastest, cached per batch shape.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np
import torch

from . import _lib
from .banded import BandedMatrix, _prefix, _ptr, _stream


def lpt_order(n, kl, ku, nrhs) -> np.ndarray:
    """System indices, most expensive first (factor + solve flop estimate)."""
    n, kl, ku, nrhs = (np.asarray(v, dtype=np.int64) for v in (n, kl, ku, nrhs))
    cost = n * (2 * kl * (kl + ku) + kl) + nrhs * 2 * n * (2 * kl + ku + 1)
    return np.argsort(-cost, kind="stable").astype(np.int32)


class Schedule(ctypes.Structure):
    """bm_gb_schedule: order[0..n_wide) solved by a CTA of `warps` warps each, the rest
    one per warp; the kl/ku bounds size each part's shared memory."""

    _fields_ = [("n_wide", ctypes.c_int64), ("warps", ctypes.c_int64), ("wide_kl", ctypes.c_int64),
                ("wide_ku", ctypes.c_int64), ("narrow_kl", ctypes.c_int64), ("narrow_ku", ctypes.c_int64)]


def schedule_order(n, kl, ku, nrhs, narrow_cols: int):
    """(order, n_wide): systems with kl+ku+1 > narrow_cols first, each part most
    expensive first."""
    n, kl, ku, nrhs = (np.asarray(v, dtype=np.int64) for v in (n, kl, ku, nrhs))
    cost = n * (2 * kl * (kl + ku) + kl) + nrhs * 2 * n * (2 * kl + ku + 1)
    wide = (kl + ku + 1) > narrow_cols
    iw, inr = np.nonzero(wide)[0], np.nonzero(~wide)[0]
    order = np.concatenate([iw[np.argsort(-cost[iw], kind="stable")], inr[np.argsort(-cost[inr], kind="stable")]])
    return order.astype(np.int32), int(len(iw))


# Candidate schedules the autotuner times: CTA width x narrow/wide split (band columns).
TUNE_WARPS = (4, 8)
TUNE_NARROW_COLS = (0, 8, 16, 24, 32, 48, 64, 96, 1 << 30)
_TUNED: dict = {}


class BandedBatch:
    """A batch of square banded systems A_s x_s = b_s with device-resident storage."""

    def __init__(self, n, kl, ku, nrhs, dtype=torch.float64, device="cuda"):
        self.count = len(n)
        self.n = np.asarray(n, dtype=np.int64)
        self.kl = np.asarray(kl, dtype=np.int64)
        self.ku = np.asarray(ku, dtype=np.int64)
        self.nrhs = np.asarray(nrhs, dtype=np.int64)
        self.dtype, self.device = dtype, torch.device(device)
        self.ldab = 2 * self.kl + self.ku + 1
        self.ab_off = np.concatenate([[0], np.cumsum(self.ldab * self.n)[:-1]]).astype(np.int64)
        self.b_off = np.concatenate([[0], np.cumsum(self.n * self.nrhs)[:-1]]).astype(np.int64)
        self.ip_off = np.concatenate([[0], np.cumsum(self.n)[:-1]]).astype(np.int64)
        self.AB = torch.zeros(int((self.ldab * self.n).sum()), dtype=dtype, device=self.device)
        self.B = torch.zeros(int((self.n * self.nrhs).sum()), dtype=dtype, device=self.device)
        self.ipiv = torch.zeros(int(self.n.sum()), dtype=torch.int64, device=self.device)
        self.info = torch.zeros(self.count, dtype=torch.int64, device=self.device)
        desc = np.stack([self.n, self.kl, self.ku, self.nrhs, self.ab_off, self.ldab, self.b_off, self.n,
                         self.ip_off], axis=1).astype(np.int64)
        self.descs = torch.from_numpy(np.ascontiguousarray(desc)).to(self.device)
        self.order = torch.from_numpy(lpt_order(self.n, self.kl, self.ku, self.nrhs)).to(self.device)
        self.counter = torch.zeros(4, dtype=torch.int32, device=self.device)  # work queues (4 for solve_mixed)
        self.max_kl = int(self.kl.max()) if self.count else 0
        self.max_ku = int(self.ku.max()) if self.count else 0
        self.schedule = None  # None: the single-part entry points (bm_*gbsv_batched)
        self.tuned = {}

    # -- launch schedule and its autotuner ------------------------------------------------
    def set_schedule(self, warps: int = 4, narrow_cols: int | None = None) -> None:
        """Use the two-part schedule: systems with more than ``narrow_cols`` band columns
        go to CTAs of ``warps`` warps, the rest to single warps.  ``narrow_cols=None``
        returns to the single-part entry points."""
        if narrow_cols is None:
            self.schedule = None
            self.order = torch.from_numpy(lpt_order(self.n, self.kl, self.ku, self.nrhs)).to(self.device)
            return
        order, n_wide = schedule_order(self.n, self.kl, self.ku, self.nrhs, narrow_cols)
        w, nr = order[:n_wide], order[n_wide:]
        mx = lambda a, idx: int(a[idx].max()) if len(idx) else 0
        self.schedule = Schedule(n_wide, int(warps), mx(self.kl, w), mx(self.ku, w), mx(self.kl, nr), mx(self.ku, nr))
        self.order = torch.from_numpy(order).to(self.device)

    def _key(self, mode: str):
        return (mode, str(self.dtype), self.count, self.n.tobytes(), self.kl.tobytes(), self.ku.tobytes(),
                self.nrhs.tobytes())

    def tune(self, mode: str = "plain", reps: int = 1, **solve_kw) -> dict:
        """Autotuner: time every candidate schedule (CTA width x narrow/wide split) on
        this batch with CUDA events and keep the fastest; results are cached per batch
        shape and mode ("plain" = factor_solve, "mixed" = solve_mixed).  The batch's
        matrices and right-hand sides are restored afterwards.  Returns
        {"warps", "narrow_cols", "ms", "candidates": [...]}."""
        key = self._key(mode)
        if key in _TUNED:
            best = _TUNED[key]
            self.set_schedule(best["warps"], best["narrow_cols"])
            self.tuned[mode] = best
            return best
        AB0, B0 = self.AB.clone(), self.B.clone()
        run = self.factor_solve if mode == "plain" else (lambda: self.solve_mixed(**solve_kw))
        widths = sorted({min(c, int((self.kl + self.ku + 1).max())) for c in TUNE_NARROW_COLS} | {0})
        results, t_start = [], time.time()
        for warps in TUNE_WARPS:
            for cols in widths:
                try:
                    self.set_schedule(warps, cols)
                    ts = []
                    for _ in range(reps + 1):
                        if mode == "plain":
                            self.AB.copy_(AB0)
                            self.B.copy_(B0)
                        e0 = torch.cuda.Event(enable_timing=True)
                        e1 = torch.cuda.Event(enable_timing=True)
                        e0.record()
                        run()
                        e1.record()
                        torch.cuda.synchronize()
                        ts.append(e0.elapsed_time(e1))
                    results.append({"warps": warps, "narrow_cols": cols, "ms": min(ts[1:] or ts)})
                except _lib.BandedGPUError:
                    continue  # the schedule's shared memory does not fit
        self.AB.copy_(AB0)
        self.B.copy_(B0)
        best = min(results, key=lambda r: r["ms"])
        best = dict(best, candidates=results, tune_s=time.time() - t_start)
        _TUNED[key] = best
        self.set_schedule(best["warps"], best["narrow_cols"])
        self.tuned[mode] = best
        return best

    # -- views of one system's storage -------------------------------------------------
    def band(self, s: int) -> BandedMatrix:
        """System s's gbtrf storage as a BandedMatrix with bandwidths (kl, kl+ku)."""
        n, ld, off = int(self.n[s]), int(self.ldab[s]), int(self.ab_off[s])
        data = self.AB[off: off + ld * n].view(n, ld).t()
        return BandedMatrix(data, n, int(self.kl[s]), int(self.kl[s] + self.ku[s]))

    def matrix_band(self, s: int) -> torch.Tensor:
        """System s's (kl+ku+1) x n band of A inside its gbtrf storage (rows kl..)."""
        return self.band(s).data[int(self.kl[s]):, :]

    def rhs(self, s: int) -> torch.Tensor:
        n, k, off = int(self.n[s]), int(self.nrhs[s]), int(self.b_off[s])
        return self.B[off: off + n * k].view(k, n).t()

    def pivots(self, s: int) -> torch.Tensor:
        off = int(self.ip_off[s])
        return self.ipiv[off: off + int(self.n[s])]

    # -- the launch ---------------------------------------------------------------------
    def factor_solve(self, stream=None) -> None:
        """Factor every system in place and overwrite its right-hand sides with the solution."""
        st = ctypes.c_void_p(stream) if stream is not None else _stream(self.device)
        if self.schedule is not None:
            _lib.call(f"bm_{_prefix(self.dtype)}gbsv_batched_sched", self.count, _ptr(self.descs), _ptr(self.order),
                      ctypes.byref(self.schedule), _ptr(self.AB), _ptr(self.ipiv), _ptr(self.B), _ptr(self.info),
                      _ptr(self.counter), st)
            return
        _lib.call(f"bm_{_prefix(self.dtype)}gbsv_batched", self.count, _ptr(self.descs), _ptr(self.order),
                  _ptr(self.AB), _ptr(self.ipiv), _ptr(self.B), _ptr(self.info), _ptr(self.counter), self.max_kl,
                  self.max_ku, st)

    def solve_mixed(self, tol: float = 1e-10, maxit: int = 30, stream=None) -> torch.Tensor:
        """FP32 factorization + FP64-residual iterative refinement (bm_dsgbsv_batched).

        The FP64 band in ``AB`` and the right-hand sides in ``B`` are left untouched; the
        solutions go to ``X`` (returned), the corrections taken per system to ``iters``
        and the final backward errors to ``berr``.  Requires a batch of Float64 storage.
        """
        if self.dtype != torch.float64:
            raise TypeError("solve_mixed refines to Float64: build the batch with dtype=torch.float64")
        if not hasattr(self, "X"):
            self.X = torch.zeros_like(self.B)
            self.AB32 = torch.zeros(self.AB.numel(), dtype=torch.float32, device=self.device)
            self.R32 = torch.zeros(self.B.numel(), dtype=torch.float32, device=self.device)
            self.iters = torch.zeros(self.count, dtype=torch.int32, device=self.device)
            self.berr = torch.zeros(self.count, dtype=torch.float64, device=self.device)
        st = ctypes.c_void_p(stream) if stream is not None else _stream(self.device)
        if self.schedule is not None:
            _lib.call("bm_dsgbsv_batched_sched", self.count, _ptr(self.descs), _ptr(self.order),
                      ctypes.byref(self.schedule), _ptr(self.AB), _ptr(self.B), _ptr(self.X), _ptr(self.ipiv),
                      _ptr(self.info), _ptr(self.AB32), _ptr(self.R32), _ptr(self.iters), _ptr(self.berr),
                      _ptr(self.counter), ctypes.c_double(tol), int(maxit), st)
            return self.X
        _lib.call("bm_dsgbsv_batched", self.count, _ptr(self.descs), _ptr(self.order), _ptr(self.AB), _ptr(self.B),
                  _ptr(self.X), _ptr(self.ipiv), _ptr(self.info), _ptr(self.AB32), _ptr(self.R32), _ptr(self.iters),
                  _ptr(self.berr), _ptr(self.counter), ctypes.c_double(tol), int(maxit), self.max_kl, self.max_ku, st)
        return self.X

    def solution(self, s: int) -> torch.Tensor:
        """System s's solution from solve_mixed (n x nrhs view of X)."""
        n, k, off = int(self.n[s]), int(self.nrhs[s]), int(self.b_off[s])
        return self.X[off: off + n * k].view(k, n).t()

    def make_plan(self, mode: str = "plain") -> "Plan":
        """A library-owned plan (bm_plan_create): the autotuned schedule of this batch for the
        plain ("plain") or refined ("mixed") solve, timed on a copy of the batch."""
        return Plan(self, mode)

    def capture(self) -> torch.cuda.CUDAGraph:
        """Capture factor_solve in a CUDA graph (call once eagerly first for device set-up)."""
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.factor_solve()
        return g


class Plan:
    """bm_plan: the batch's autotuned schedule and its device workspace, owned by the
    library (the C-ABI counterpart of BandedBatch.tune).  Release with close()."""

    def __init__(self, batch: BandedBatch, mode: str = "plain"):
        if mode not in ("plain", "mixed") or batch.dtype != torch.float64:
            raise ValueError("plans cover the Float64 plain and refined batched solves")
        self.batch, self.mode = batch, mode
        self.handle = ctypes.c_void_p()
        host = np.ascontiguousarray(batch.descs.cpu().numpy())
        _lib.call("bm_plan_create", ctypes.byref(self.handle), batch.count, ctypes.c_void_p(host.ctypes.data),
                  _ptr(batch.descs), 0 if mode == "plain" else 1, _ptr(batch.AB), _ptr(batch.B), _stream(batch.device))
        sched, ms, cand = Schedule(), ctypes.c_double(), ctypes.c_int64()
        _lib.call("bm_plan_schedule", self.handle, ctypes.byref(sched), ctypes.byref(ms), ctypes.byref(cand))
        self.schedule, self.tuned_ms, self.candidates = sched, ms.value, cand.value

    def execute(self, tol: float = 1e-10, maxit: int = 30, stream=None) -> None:
        """The scheduled solve of the plan's batch (factor_solve / solve_mixed semantics)."""
        b = self.batch
        st = ctypes.c_void_p(stream) if stream is not None else _stream(b.device)
        if self.mode == "plain":
            _lib.call("bm_plan_execute_dgbsv", self.handle, _ptr(b.descs), _ptr(b.AB), _ptr(b.ipiv), _ptr(b.B),
                      _ptr(b.info), st)
            return
        if not hasattr(b, "X"):
            b.solve_mixed(tol, maxit)  # allocates the refined solve's buffers once
        _lib.call("bm_plan_execute_dsgbsv", self.handle, _ptr(b.descs), _ptr(b.AB), _ptr(b.B), _ptr(b.X),
                  _ptr(b.ipiv), _ptr(b.info), _ptr(b.AB32), _ptr(b.R32), _ptr(b.iters), _ptr(b.berr),
                  ctypes.c_double(tol), int(maxit), st)

    def close(self) -> None:
        if self.handle:
            _lib.call("bm_plan_destroy", self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
