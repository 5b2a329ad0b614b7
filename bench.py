#!/usr/bin/env python3
"""Benchmark of the banded hot path on one GB300 (or N replicas under torchrun).

Workload (one "step"): the bandwidth-bound sweep -- y = A*x (gbmv) for a square
n = 2^24 band with l = u in {1, 8, 32}, in Float32 and Float64 band storage,
entries uniform(-1,1), x randn; plus banded_mul of two n = 2^20, l = u = 16
matrices (result bandwidth (32,32)) in both precisions.  Every operand set is
larger than the 129 MB L2, so timed iterations stream from HBM.

value  = algorithmic bytes of all kernels of a step / device time of a step (GB/s)
e2e    = the same bytes / time of the same step through the public API with
         host buffers (pinned host -> device copies of A, B and x, and device
         -> host copies of y and C, inside the timed region)
--impl reference times the reference's CPU path (OpenBLAS dgbmv/sgbmv, the
routine BandedMatrices.jl ccalls for A*x, and the _gbmm! column loop over it)
on the host cores.
"""
from __future__ import annotations

import argparse
import ctypes
import glob
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "banded LU+solve systems/s & gbmv GB/s vs plain FP64 GPU at 1e-10 backward err"
GBMV_CASES = [("f32", 1), ("f32", 8), ("f32", 32), ("f64", 1), ("f64", 8), ("f64", 32)]
N_GBMV = 1 << 24
N_GBMM, LU_GBMM = 1 << 20, 16
WORKLOAD = ("gbmv y=A*x, n=2^24 square, l=u in {1,8,32}, f32+f64, uniform(-1,1) band, randn x; "
            "banded_mul n=2^20 l=u=16 -> (32,32), f32+f64")


def gbmv_bytes(n, l, u, s):
    # band (l+u+1)*n + x n + y n (beta = 0: y written only)
    return s * n * (l + u + 1 + 2)


def gbmv_fmas(n, l, u):
    """Multiply-adds of y = A*x for a square n x n band (every in-matrix entry once)."""
    return n * (l + u + 1) - l * (l + 1) // 2 - u * (u + 1) // 2


def gbmm_fmas(n, l, u):
    """Multiply-adds of C = A*B for two square n x n (l,u) bands (interior count per column)."""
    w = l + u + 1
    return n * w * w


def gbmm_bytes(n, l, u, s):
    # A and B (l+u+1)*n each, C (2l+2u+1)*n written
    return s * n * ((l + u + 1) * 2 + (2 * l + 2 * u + 1))


# --------------------------------------------------------------------------- CPU (OpenBLAS)
def _openblas():
    import scipy

    libdir = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    L = ctypes.CDLL(glob.glob(os.path.join(libdir, "libscipy_openblas*.so"))[0])
    i, d, f, p = ctypes.c_int, ctypes.c_double, ctypes.c_float, ctypes.c_void_p
    L.scipy_cblas_dgbmv.argtypes = [i, i, i, i, i, i, d, p, i, p, i, d, p, i]
    L.scipy_cblas_sgbmv.argtypes = [i, i, i, i, i, i, f, p, i, p, i, f, p, i]
    L.scipy_cblas_dgbmv.restype = L.scipy_cblas_sgbmv.restype = None
    L.scipy_openblas_get_num_threads.restype = ctypes.c_int
    return L


def _fill(a, kind: str, seed: int, threads: int = 16) -> None:
    """Fill a contiguous numpy array in place with uniform(-1,1) ('u') or standard normal
    ('n') values, in parallel chunks, each with its own seeded PCG64 stream (numpy's
    generators release the GIL while they fill)."""
    import concurrent.futures as cf

    import numpy as np

    flat = a.reshape(-1, order="F" if a.flags.f_contiguous else "C")
    chunks = np.array_split(np.arange(flat.size), threads)

    def work(i):
        if not len(chunks[i]):
            return
        v = flat[chunks[i][0]: chunks[i][-1] + 1]
        rng = np.random.default_rng([seed, i])
        if kind == "u":
            rng.random(out=v, dtype=v.dtype)
            v *= 2
            v -= 1
        else:
            rng.standard_normal(out=v, dtype=v.dtype)

    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(work, range(threads)))


def cpu_operands():
    """Host operands of the sweep at the full sizes: the six gbmv cases at n = 2^24 and
    the two banded_mul cases at n = 2^20 (uniform(-1,1) bands, randn x)."""
    import numpy as np

    gbmv = []
    for k, (dt, lu) in enumerate(GBMV_CASES):
        nt = np.float32 if dt == "f32" else np.float64
        A = np.empty((2 * lu + 1, N_GBMV), dtype=nt, order="F")
        _fill(A, "u", 100 + k)
        x = np.empty(N_GBMV, dtype=nt)
        _fill(x, "n", 200 + k)
        gbmv.append((dt, lu, A, x, np.zeros(N_GBMV, dtype=nt)))
    mm = []
    for k, dt in enumerate(("f32", "f64")):
        nt = np.float32 if dt == "f32" else np.float64
        A = np.empty((2 * LU_GBMM + 1, N_GBMM), dtype=nt, order="F")
        B = np.empty((2 * LU_GBMM + 1, N_GBMM), dtype=nt, order="F")
        _fill(A, "u", 300 + k)
        _fill(B, "u", 400 + k)
        mm.append((dt, A, B, np.zeros((4 * LU_GBMM + 1, N_GBMM), dtype=nt, order="F")))
    return gbmv, mm


def cpu_sweep(steps: int, warmup: int, one_thread_steps: int = 3):
    """The reference's CPU path for the sweep, on the host cores, at the full sizes:
    OpenBLAS {s,d}gbmv (the routine BandedMatrices.jl ccalls for A*x) for the six
    n = 2^24 cases, and the _gbmm! column loop (gbmm.jl:296-340, restated in C over the
    same OpenBLAS gbmv) for the two n = 2^20 products.  `warmup` untimed steps, then
    `steps` timed ones with all OpenBLAS threads; value = bytes of a step / median step
    time.  Then `one_thread_steps` steps with OpenBLAS on one thread, reported beside."""
    import numpy as np

    L = _openblas()
    threads = int(L.scipy_openblas_get_num_threads())
    gbmv, mm = cpu_operands()

    import oracle  # CPU-baseline leg: the _gbmm! column loop restated in C over OpenBLAS gbmv

    orl = oracle.lib()
    fptr = {"f32": ctypes.cast(L.scipy_cblas_sgbmv, ctypes.c_void_p).value,
            "f64": ctypes.cast(L.scipy_cblas_dgbmv, ctypes.c_void_p).value}
    step_bytes = (sum(gbmv_bytes(N_GBMV, lu, lu, A.itemsize) for _, lu, A, _, _ in gbmv)
                  + sum(gbmm_bytes(N_GBMM, LU_GBMM, LU_GBMM, A.itemsize) for _, A, _, _ in mm))

    def one_step():
        t0 = time.perf_counter()
        for dt, lu, A, x, y in gbmv:
            fn = L.scipy_cblas_sgbmv if dt == "f32" else L.scipy_cblas_dgbmv
            fn(102, 111, N_GBMV, N_GBMV, lu, lu, 1.0, A.ctypes.data, 2 * lu + 1, x.ctypes.data, 1, 0.0,
               y.ctypes.data, 1)
        t1 = time.perf_counter()
        for dt, A, B, C in mm:
            fn = orl.or_sgbmm_percol_cblas if dt == "f32" else orl.or_dgbmm_percol_cblas
            T = ctypes.c_float if dt == "f32" else ctypes.c_double
            w = 2 * LU_GBMM + 1
            fn(ctypes.c_void_p(fptr[dt]), N_GBMM, N_GBMM, N_GBMM, LU_GBMM, LU_GBMM, LU_GBMM, LU_GBMM, T(1.0),
               ctypes.c_void_p(A.ctypes.data), w, ctypes.c_void_p(B.ctypes.data), w, T(0.0),
               ctypes.c_void_p(C.ctypes.data), 2 * w - 1)
        t2 = time.perf_counter()
        return t1 - t0, t2 - t1

    def run(k, w):
        for _ in range(w):
            one_step()
        return [one_step() for _ in range(max(1, k))]

    s_all = run(steps, warmup)
    s_one = []
    if one_thread_steps > 0 and hasattr(L, "scipy_openblas_set_num_threads"):
        L.scipy_openblas_set_num_threads(1)
        try:
            s_one = run(one_thread_steps, 0)
        finally:
            L.scipy_openblas_set_num_threads(threads)
    gb_bytes = step_bytes - sum(gbmm_bytes(N_GBMM, LU_GBMM, LU_GBMM, A.itemsize) for _, A, _, _ in mm)
    med = statistics.median(a + b for a, b in s_all)
    out = {
        "value": step_bytes / med / 1e9,
        "sec_per_step": med,
        "sec_total": sum(a + b for a, b in s_all),
        "steps": len(s_all),
        "warmup": warmup,
        "gbmv_GBps": gb_bytes / statistics.median(a for a, _ in s_all) / 1e9,
        "gbmm_GBps": (step_bytes - gb_bytes) / statistics.median(b for _, b in s_all) / 1e9,
        "threads": threads,
        "host_cores": os.cpu_count(),
        "sample": (f"the full sweep (gbmv n=2^24 l=u in {{1,8,32}} f32+f64; banded_mul n=2^20 l=u=16 f32+f64) on "
                   f"the host: OpenBLAS {{s,d}}gbmv via SciPy's bundled libscipy_openblas (the BLAS routine "
                   f"BandedMatrices.jl ccalls; Julia absent) and the _gbmm! column loop restated in C over it; "
                   f"median of {len(s_all)} steps after {warmup} warm-up, {threads} threads"),
    }
    if s_one:
        out["one_thread"] = {"value": step_bytes / statistics.median(a + b for a, b in s_one) / 1e9,
                             "steps": len(s_one),
                             "gbmv_GBps": gb_bytes / statistics.median(a for a, _ in s_one) / 1e9,
                             "gbmm_GBps": (step_bytes - gb_bytes) / statistics.median(b for _, b in s_one) / 1e9}
    del np
    return out


def bench_config(world: int) -> dict:
    """The `config` object of both arms' JSON lines (identical, so the lines compare)."""
    return {"workload": WORKLOAD, "l2": "every operand set > 129 MB L2 (no flush needed)",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"bm_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [v.strip() for v in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------- GPU
def cpu_lu_baselines():
    """The reference's CPU path for the LU/QR/PDE workloads on the host cores: OpenBLAS
    dgbtrf + dgbtrs through SciPy (the LAPACK routines lu!/ldiv! ccall; Julia absent),
    all OpenBLAS threads, seeded NumPy inputs of the same shapes; bounded samples are
    scaled by their share of the work and say so.  QR: the _banded_qr! restatement in C
    (one thread, as the reference's Julia loop)."""
    import numpy as np
    from scipy.linalg import lapack

    L = _openblas()
    threads = int(L.scipy_openblas_get_num_threads())
    rng = np.random.default_rng(7)

    def gb(n, kl, ku, shift):
        ab = np.zeros((2 * kl + ku + 1, n), order="F")
        ab[kl:, :] = rng.standard_normal((kl + ku + 1, n))
        ab[kl + ku, :] += shift
        return ab

    def lu_solve(n, kl, ku, shift, nrhs=1, trans=0):
        ab = gb(n, kl, ku, shift)
        b = rng.standard_normal((n, nrhs))
        t0 = time.perf_counter()
        lub, piv, info = lapack.dgbtrf(ab, kl, ku, overwrite_ab=1)
        t1 = time.perf_counter()
        x, info2 = lapack.dgbtrs(lub, kl, ku, b, piv, trans=trans)
        t2 = time.perf_counter()
        return t1 - t0, t2 - t1

    out = {"threads": threads, "kind": "reference", "impl": "OpenBLAS dgbtrf/dgbtrs via SciPy (stand-in for Julia's ccall)"}
    f, s_ = lu_solve(10000, 4, 3, 10.0)
    out["config1_lu_solve_ms"] = (f + s_) * 1e3
    # 4096 uneven systems: a sample of 512 of them, scaled by its share of the flops
    n, kl, ku, nrhs = batched_config()
    idx = np.random.default_rng(1).choice(len(n), 512, replace=False)
    cost = n * (2 * kl * (kl + ku) + kl) + nrhs * 2 * n * (2 * kl + ku + 1)
    tot = 0.0
    for s in idx:
        f, s_ = lu_solve(int(n[s]), int(kl[s]), int(ku[s]), 2.0 * (kl[s] + ku[s]), int(nrhs[s]))
        tot += f + s_
    t_all = tot * cost.sum() / cost[idx].sum()
    out["batched_4096_ms"] = t_all * 1e3
    out["batched_systems_per_s"] = len(n) / t_all
    out["batched_sample"] = "512 of the 4096 systems (seeded), time scaled by the flop share"
    f, s_ = lu_solve(1 << 20, 128, 128, 16.0)
    out["refined_config_fp64_lu_solve_ms"] = (f + s_) * 1e3
    f, s_ = lu_solve(262144, 512, 512, 4.0 * 1024, trans=0)
    out["pde_factor_ms"], out["pde_solve_ms"] = f * 1e3, s_ * 1e3
    import oracle  # CPU-baseline leg: the _banded_qr! restatement

    nq, lq = 1 << 15, 32
    D = np.zeros((3 * lq + 1, nq), order="F")
    D[lq:, :] = rng.standard_normal((2 * lq + 1, nq))
    t0 = time.perf_counter()
    oracle.gbqrf(nq, nq, lq, 2 * lq, D)
    out["qr_factor_n2e18_ms"] = (time.perf_counter() - t0) * 1e3 * (1 << 18) / nq
    out["qr_sample"] = "n = 2^15, l = u = 32, scaled by columns to n = 2^18"
    return out


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _traffic(name):
    """DRAM bytes per launch of a kernel from a committed ncu summary (profiles/*.md)."""
    for f in glob.glob(os.path.join(ROOT, "profiles", "*.md")):
        for line in open(f):
            if line.startswith(f"traffic[{name}]"):
                try:
                    return float(line.split("=")[1].split()[0])
                except (IndexError, ValueError):
                    pass
    return None


def run_gpu(args, rank, world):
    import torch
    import __graft_entry__ as ge

    bm = ge.package()
    bm.load_library()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)
    g = torch.Generator(device=dev)
    g.manual_seed(1000 + rank)

    gb = []  # (label, A, x, y, bytes)
    for dt_name, lu in GBMV_CASES:
        dt = torch.float32 if dt_name == "f32" else torch.float64
        A = bm.BandedMatrix(bm.band_storage(2 * lu + 1, N_GBMV, dt, dev), N_GBMV, lu, lu)
        A.data.uniform_(-1.0, 1.0, generator=g)
        x = torch.randn(N_GBMV, dtype=dt, device=dev, generator=g)
        y = torch.empty(N_GBMV, dtype=dt, device=dev)
        gb.append((f"gbmv_{dt_name}_l{lu}", A, x, y, gbmv_bytes(N_GBMV, lu, lu, A.data.element_size())))
    mm = []
    if hasattr(bm, "banded_mul_"):
        for dt_name in ("f32", "f64"):
            dt = torch.float32 if dt_name == "f32" else torch.float64
            A = bm.BandedMatrix(bm.band_storage(33, N_GBMM, dt, dev), N_GBMM, 16, 16)
            B = bm.BandedMatrix(bm.band_storage(33, N_GBMM, dt, dev), N_GBMM, 16, 16)
            A.data.uniform_(-1.0, 1.0, generator=g)
            B.data.uniform_(-1.0, 1.0, generator=g)
            C = bm.BandedMatrix(bm.band_storage(65, N_GBMM, dt, dev), N_GBMM, 32, 32)
            mm.append((f"gbmm_{dt_name}_l16", A, B, C, gbmm_bytes(N_GBMM, 16, 16, A.data.element_size())))

    # Each case is captured once as a CUDA graph (the C ABI only enqueues, so the
    # launches capture cleanly); the timed region replays the graphs back to back.
    calls = []
    for lab, A, x, y, nb in gb:
        calls.append((lab, (lambda A=A, x=x, y=y: bm.gbmv("N", 1.0, A, x, 0.0, y)), nb))
    for lab, A, B, C, nb in mm:
        calls.append((lab, (lambda A=A, B=B, C=C: bm.banded_mul_(C, A, B, 1.0, 0.0)), nb))
    for _, fn, _ in calls:
        fn()  # first call: per-device set-up outside capture
    torch.cuda.synchronize()
    lib = bm._lib.load()
    graphs = []
    n_launch = 0  # library kernels per step, counted by the library itself
    for lab, fn, nb in calls:
        gr = torch.cuda.CUDAGraph()
        c0 = lib.bm_launch_count()
        with torch.cuda.graph(gr):
            fn()
        n_launch += lib.bm_launch_count() - c0
        graphs.append((lab, gr, nb))
    ev = {lab: [] for lab, _, _ in graphs}

    def step():
        for _, gr, _ in graphs:
            gr.replay()

    with ClockSampler(dev.index) as clk:
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0.record(stream)
        for _ in range(args.steps):
            step()
        t1.record(stream)
        torch.cuda.synchronize()
        # Per-case figures: each case's graph replayed back to back, the first replay
        # untimed.  A kernel then inherits only its own write-backs of dirty L2 lines;
        # inside the step it inherits the previous case's (up to ~100 MB after the
        # Float64 product), which the sweep step total above includes.
        for lab, gr, _ in graphs:
            gr.replay()
            for _ in range(args.steps):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                gr.replay()
                e1.record(stream)
                ev[lab].append((e0, e1))
        torch.cuda.synchronize()
    ms = t0.elapsed_time(t1)
    if world > 1:
        tt = torch.tensor([ms], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.barrier()
        ms = float(tt.item())
    step_bytes = sum(nb for _, _, nb in graphs)
    value = world * step_bytes * args.steps / (ms / 1e3) / 1e9

    per_case = []
    for lab, _, nb in graphs:
        t_ms = statistics.mean(a.elapsed_time(b) for a, b in ev[lab])
        per_case.append({"case": lab, "GBps": nb / (t_ms / 1e3) / 1e9, "ms": t_ms, "bytes": nb})
    peak, peak_kind = _peaks()
    fma_peak = {}
    for eb in (8, 4):  # the FP64 / FP32 fma roofs, probed on this GPU
        v = ctypes.c_double(0.0)
        bm._lib.check(lib.bm_probe_fma_rate(eb, ctypes.byref(v), ctypes.c_void_p(stream.cuda_stream)), "probe")
        fma_peak[eb] = v.value
    for c in per_case:
        c["frac_of_hbm"] = c["GBps"] / peak
        lu = int(c["case"].split("_l")[1])
        f = gbmv_fmas(N_GBMV, lu, lu) if c["case"].startswith("gbmv") else gbmm_fmas(N_GBMM, lu, lu)
        c["fma_per_s"] = f / (c["ms"] / 1e3)
        c["frac_of_fma_roof"] = c["fma_per_s"] / fma_peak[8 if "_f64_" in c["case"] else 4]
    dom = max(per_case, key=lambda c: c["ms"])
    traffic = _traffic(dom["case"])

    # e2e through the public API with host buffers
    e2e = None
    if rank == 0 or world > 1:
        e2e = run_e2e(bm, gb, mm, dev, stream, args.steps)
    out = None
    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (torch Philox, seeded)",
            "config": bench_config(world),
            "roofline": {"bound": "hbm", "kernel": dom["case"], "achieved": dom["GBps"], "peak": peak,
                         "unit": "GB/s", "frac": dom["GBps"] / peak, "traffic": traffic,
                         "peak_source": f"{peak_kind} hbm_gbs",
                         # the Float64 cases are bounded first by the FP64 pipe (probed fma rate)
                         "compute_roof": {"unit": "fma/s", "achieved": dom["fma_per_s"],
                                          "peak": fma_peak[8 if "_f64_" in dom["case"] else 4],
                                          "frac": dom["frac_of_fma_roof"],
                                          "peak_source": "probed (bm_probe_fma_rate)"}},
            "sweep": per_case,
            "e2e": e2e,
            "gpu_launches": n_launch * args.steps,
            "fma_roofs": {"f64": fma_peak[8], "f32": fma_peak[4]},
            "clocks": clk.summary(),
        }
    return out


def run_e2e(bm, gb, mm, dev, stream, steps):
    """Same step through the public API with pinned host inputs/outputs; copies are timed."""
    import torch

    host = []
    h2d = d2h = 0
    for lab, A, x, y, nb in gb:
        hA = torch.empty(A.data.shape[1], A.lda, dtype=A.dtype, pin_memory=True)
        hA.copy_(A.data.t())
        hx = torch.empty(x.shape, dtype=x.dtype, pin_memory=True)
        hx.copy_(x)
        hy = torch.empty(y.shape, dtype=y.dtype, pin_memory=True)
        host.append(("gbmv", A, hA, x, hx, y, hy, nb))
        h2d += hA.numel() * hA.element_size() + hx.numel() * hx.element_size()
        d2h += hy.numel() * hy.element_size()
    for lab, A, B, C, nb in mm:
        hA = torch.empty(A.data.shape[1], A.lda, dtype=A.dtype, pin_memory=True)
        hA.copy_(A.data.t())
        hB = torch.empty(B.data.shape[1], B.lda, dtype=B.dtype, pin_memory=True)
        hB.copy_(B.data.t())
        hC = torch.empty(C.data.shape[1], C.lda, dtype=C.dtype, pin_memory=True)
        host.append(("gbmm", A, hA, B, hB, C, hC, nb))
        h2d += 2 * hA.numel() * hA.element_size()
        d2h += hC.numel() * hC.element_size()
    nbytes = sum(h[-1] for h in host)
    # Three streams: host->device copies, the library calls, device->host copies.  Case
    # k+1's inputs stream in while case k computes and returns its result; a case's
    # device buffers are refilled only after the previous step read its result back.
    s_in, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    ev_in = [torch.cuda.Event() for _ in host]
    ev_done = [torch.cuda.Event() for _ in host]
    ev_out = [torch.cuda.Event() for _ in host]
    for e in ev_out:
        e.record(stream)

    def step():
        for i, (kind, A, hA, X, hX, Y, hY, nb) in enumerate(host):
            s_in.wait_event(ev_out[i])
            with torch.cuda.stream(s_in):
                A.data.t().copy_(hA, non_blocking=True)
                if kind == "gbmv":
                    X.copy_(hX, non_blocking=True)
                else:
                    X.data.t().copy_(hX, non_blocking=True)
                ev_in[i].record(s_in)
            stream.wait_event(ev_in[i])
            if kind == "gbmv":
                bm.gbmv("N", 1.0, A, X, 0.0, Y)
            else:
                bm.banded_mul_(Y, A, X, 1.0, 0.0)
            ev_done[i].record(stream)
            s_out.wait_event(ev_done[i])
            with torch.cuda.stream(s_out):
                hY.copy_(Y if kind == "gbmv" else Y.data.t(), non_blocking=True)
                ev_out[i].record(s_out)
        for e in ev_out:  # the step ends when every result is back on the host
            stream.wait_event(e)

    step()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    s_in.wait_event(t0)  # no copy of the timed steps starts before t0
    for _ in range(steps):
        step()
    t1.record(stream)
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / steps
    return {"value": nbytes / (ms / 1e3) / 1e9, "unit": "GB/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "ms_per_step": ms, "steps": steps}


# --------------------------------------------------------------------- other workloads
def _timed(fn, stream, reps=1, restore=None):
    import torch

    ts = []
    for _ in range(reps):
        if restore:
            restore()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return min(ts)


def batched_config(n_sys=4096, seed=3):
    """4096 systems: n log-uniform in [256,16384], l,u uniform in [1,64], 1-8 right-hand sides."""
    import numpy as np

    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(np.log(256), np.log(16384), n_sys)).astype(np.int64)
    kl = rng.integers(1, 65, n_sys)
    ku = rng.integers(1, 65, n_sys)
    nrhs = rng.integers(1, 9, n_sys)
    return n, kl, ku, nrhs


def run_batched(bm, dev, stream):
    """Plain FP64 factor+solve vs FP32-factor/FP64-refined solve of the same batch."""
    import numpy as np
    import torch

    n, kl, ku, nrhs = batched_config()
    batch = bm.BandedBatch(n, kl, ku, nrhs, torch.float64, dev)
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    for s in range(batch.count):
        mb = batch.matrix_band(s)
        mb.normal_(generator=g)
        mb[int(ku[s])] += 2.0 * (kl[s] + ku[s])
        batch.rhs(s).normal_(generator=g)
    AB0, B0 = batch.AB.clone(), batch.B.clone()

    def restore():
        batch.AB.copy_(AB0)
        batch.B.copy_(B0)

    restore()
    tune_plain = batch.tune("plain")  # autotuner: schedule for the plain solve
    restore()
    batch.factor_solve()  # warm-up (device set-up)
    lib = bm._lib.load()
    c0 = lib.bm_launch_count()
    batch.factor_solve()
    launches_plain = lib.bm_launch_count() - c0
    restore()
    t_plain = _timed(batch.factor_solve, stream, reps=2, restore=restore)
    # backward error of the plain solutions on a sample of systems (FP64 residual on the GPU)
    berr_plain = 0.0
    for s in range(0, batch.count, 256):
        A = bm.BandedMatrix(AB0[int(batch.ab_off[s]): int(batch.ab_off[s] + batch.ldab[s] * batch.n[s])]
                            .view(int(batch.n[s]), int(batch.ldab[s])).t()[int(kl[s]):], int(n[s]), int(kl[s]),
                            int(ku[s]))
        X = batch.rhs(s)
        Bs = B0[int(batch.b_off[s]): int(batch.b_off[s] + n[s] * nrhs[s])].view(int(nrhs[s]), int(n[s])).t()
        absA = bm.BandedMatrix(A.data.abs().contiguous().t().contiguous().t(), A.m, A.l, A.u)
        an = (absA @ torch.ones(A.n, dtype=torch.float64, device=dev)).max().item()
        for c in range(int(nrhs[s])):
            r = Bs[:, c].contiguous()
            bm.mul_(r, A, X[:, c].contiguous(), -1.0, 1.0)
            be = r.abs().max().item() / (an * X[:, c].abs().max().item() + Bs[:, c].abs().max().item())
            berr_plain = max(berr_plain, be)
    restore()
    tune_mixed = batch.tune("mixed", tol=1e-10, maxit=30)
    c0 = lib.bm_launch_count()
    batch.solve_mixed(1e-10, 30)
    launches_mixed = lib.bm_launch_count() - c0
    t_mixed = _timed(lambda: batch.solve_mixed(1e-10, 30), stream, reps=2)
    its = batch.iters.cpu().numpy()
    flops = float((n * (2 * kl * (kl + ku) + kl) + nrhs * 2 * n * (2 * kl + ku + 1)).sum())
    return {
        "workload": "4096 systems, n log-uniform [256,16384], l,u uniform [1,64], 1-8 RHS, randn + 2(l+u) I",
        "plain_fp64": {"ms": t_plain, "systems_per_s": batch.count / (t_plain / 1e3),
                       "gflops": flops / (t_plain / 1e3) / 1e9, "max_berr_sampled": berr_plain},
        "mixed_fp32_fp64_refined": {"ms": t_mixed, "systems_per_s": batch.count / (t_mixed / 1e3),
                                    "tol": 1e-10, "max_berr": float(batch.berr.max().item()),
                                    "iters_max": int(its.max()), "iters_mean": float(its.mean())},
        "speedup_mixed_vs_plain": t_plain / t_mixed,
        # library kernels per call; the refined call enqueues maxit correction/residual
        # pairs, which return at once after every system has converged
        "launches_per_solve": {"plain": launches_plain, "mixed": launches_mixed},
        "schedule": {"plain": {k: tune_plain[k] for k in ("warps", "narrow_cols", "ms", "tune_s")},
                     "mixed": {k: tune_mixed[k] for k in ("warps", "narrow_cols", "ms", "tune_s")},
                     "candidates_timed": len(tune_plain["candidates"]) + len(tune_mixed["candidates"])},
    }


def run_refined(bm, dev, stream):
    """One system n = 2^20, l = u = 128: randn band + 16 on the diagonal (kappa_1 ~ 1e6,
    estimated from the LU factors at n = 2^16 with the same recipe), b randn.  Float32
    LU + Float64-residual refinement to 1e-10 against the plain Float64 LU solve."""
    import torch

    def band(n, seed):
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        A = bm.BandedMatrix(bm.band_storage(257, n, torch.float64, dev), n, 128, 128)
        A.data.normal_(generator=g)
        A.data[128] += 16.0
        return A, torch.randn(n, dtype=torch.float64, device=dev, generator=g)

    Ap, _ = band(1 << 16, 20)
    Fp = bm.lu(Ap)
    kappa = float(Ap.data.abs().sum(0).max()) * Fp.inv_norm1_estimate()
    del Ap, Fp
    A, b = band(1 << 20, 21)
    out = {}
    t_ref = _timed(lambda: out.__setitem__("r", bm.solve_refined(A, b, tol=1e-10)), stream)
    x, st = out["r"]
    t_plain = _timed(lambda: out.__setitem__("p", bm.lu(A).solve(b)), stream)
    xp = out["p"]
    r = b.clone()
    bm.mul_(r, A, xp, -1.0, 1.0)
    an = float(A.data.abs().sum(0).max())
    berr_plain = float(r.abs().max()) / (an * float(xp.abs().max()) + float(b.abs().max()))
    del A, b, x, xp, r
    return {"workload": "n=2^20, l=u=128, f64 randn + 16 I (kappa_1 ~ %.1e at n=2^16), b randn" % kappa,
            "refined_ms": t_ref, "iters": int(st["iters"]), "berr": float(st["berr"]), "plain_fp64_ms": t_plain,
            "berr_plain": berr_plain, "speedup_refined_vs_plain": t_plain / t_ref}


def run_cpu_runnable(bm, dev, stream):
    """brandn(10000,10000,4,3) + 10I: A*b, A*A and A\\b latencies on the GPU."""
    import torch

    n, l, u = 10000, 4, 3
    g = torch.Generator(device=dev)
    g.manual_seed(0)
    A = bm.brandn(torch.float64, n, n, l, u, device=dev, generator=g)
    A.data[u] += 10.0
    b = torch.randn(n, dtype=torch.float64, device=dev, generator=g)
    y = torch.empty(n, dtype=torch.float64, device=dev)
    C = bm.BandedMatrix.zeros((n, n), (2 * l, 2 * u), torch.float64, dev)
    for _ in range(3):
        bm.mul_(y, A, b)
        bm.banded_mul_(C, A, A)
        x = A.solve(b)
    t_mv = _timed(lambda: bm.mul_(y, A, b), stream, reps=5)
    t_mm = _timed(lambda: bm.banded_mul_(C, A, A), stream, reps=5)
    t_sv = _timed(lambda: A.solve(b), stream, reps=5)
    return {"workload": "n=10000, (l,u)=(4,3), f64, randn + 10 I", "gbmv_us": t_mv * 1e3, "gbmm_us": t_mm * 1e3,
            "lu_solve_us": t_sv * 1e3}


def run_qr(bm, dev, stream):
    """Banded QR least-squares solve, n = 2^18, l = u = 32, with an FP64 residual check."""
    import torch

    n, l, u = 1 << 18, 32, 32
    g = torch.Generator(device=dev)
    g.manual_seed(7)
    A = bm.BandedMatrix(bm.band_storage(l + u + 1, n, torch.float64, dev), n, l, u)
    A.data.normal_(generator=g)
    b = torch.randn(n, dtype=torch.float64, device=dev, generator=g)
    F = bm.qr(A)
    out = {}
    t_f = _timed(lambda: out.__setitem__("F", bm.qr(A)), stream)
    t_s = _timed(lambda: out.__setitem__("x", out["F"].solve(b)), stream)
    x = out["x"]
    r = b.clone()
    bm.mul_(r, A, x, -1.0, 1.0)
    absA = bm.BandedMatrix(A.data.abs(), n, l, u)
    an = (absA @ torch.ones(n, dtype=torch.float64, device=dev)).max().item()
    berr = r.abs().max().item() / (an * x.abs().max().item() + b.abs().max().item())
    del F
    return {"workload": "qr(A) \\ b, n=2^18, l=u=32, f64 randn", "factor_ms": t_f, "solve_ms": t_s,
            "gflops_factor": 4.0 * n * (l + 1) * (2 * l + u) / (t_f / 1e3) / 1e9, "berr": berr}


def run_pde(bm, dev, stream, G=512):
    """Differentiated PDE solve: 5-point variable-coefficient diffusion on a G x G grid,
    x = A \\ b, L = w.x, adjoint dL/db and dL/dA; directional central difference h = 1e-6."""
    import numpy as np
    import torch

    kcell = np.exp(bm.pde.gaussian_field(G, 16.0, seed=11))
    A = bm.pde.diffusion_band(kcell, torch.float64, dev)
    n = G * G
    rng = np.random.default_rng(12)
    b = torch.from_numpy(rng.standard_normal(n)).to(dev)
    w = torch.from_numpy(rng.standard_normal(n)).to(dev)
    D = A.data.clone().requires_grad_(True)
    bt = b.clone().requires_grad_(True)
    st = {}

    def fwd():
        st["x"] = bm.banded_solve(D, bt, G, G)

    def bwd():
        (st["x"] * w).sum().backward()

    fwd()
    bwd()
    D.grad = None
    bt.grad = None
    t_f = _timed(fwd, stream)
    t_b = _timed(bwd, stream)
    h = 1e-6
    dD = torch.from_numpy(rng.standard_normal(tuple(A.data.shape))).to(dev) * (A.data != 0)
    db = torch.from_numpy(rng.standard_normal(n)).to(dev)
    L = lambda d, bb: float((bm.banded_solve(d, bb, G, G) * w).sum())
    fd = (L(A.data + h * dD, b + h * db) - L(A.data - h * dD, b - h * db)) / (2 * h)
    ad = float((D.grad * dD).sum() + (bt.grad * db).sum())
    return {"workload": f"5-point diffusion, {G}x{G} grid (n={n}, l=u={G}), exp(GRF, corr 16), f64",
            "forward_ms": t_f, "adjoint_ms": t_b, "fd_rel_err": abs(fd - ad) / max(1.0, abs(fd))}


def run_case(args):
    """One named workload, repeated --reps times (for profiler captures); prints the
    device time of each repetition.  Cases: gbmv_{f32,f64}_l{L}, gbmm_{f32,f64}_l{L},
    batched_plain, batched_mixed, lu_single_l{L}, refined_l{L}, qr_l{L}."""
    import numpy as np
    import torch
    import __graft_entry__ as ge

    bm = ge.package()
    bm.load_library()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    g = torch.Generator(device=dev)
    g.manual_seed(7)
    name = args.case
    parts = name.split("_")
    dt = torch.float32 if "f32" in parts else torch.float64
    lu = int(name.split("_l")[-1]) if "_l" in name else 0
    if parts[0] == "gbmv":
        n = args.n or N_GBMV
        A = bm.BandedMatrix(bm.band_storage(2 * lu + 1, n, dt, dev), n, lu, lu)
        A.data.uniform_(-1.0, 1.0, generator=g)
        x = torch.randn(n, dtype=dt, device=dev, generator=g)
        y = torch.empty(n, dtype=dt, device=dev)
        fn = lambda: bm.gbmv("N", 1.0, A, x, 0.0, y)
    elif parts[0] == "gbmm":
        n = args.n or N_GBMM
        A = bm.BandedMatrix(bm.band_storage(2 * lu + 1, n, dt, dev), n, lu, lu)
        B = bm.BandedMatrix(bm.band_storage(2 * lu + 1, n, dt, dev), n, lu, lu)
        A.data.uniform_(-1.0, 1.0, generator=g)
        B.data.uniform_(-1.0, 1.0, generator=g)
        C = bm.BandedMatrix(bm.band_storage(4 * lu + 1, n, dt, dev), n, 2 * lu, 2 * lu)
        fn = lambda: bm.banded_mul_(C, A, B, 1.0, 0.0)
    elif parts[0] == "batched":
        n, kl, ku, nrhs = batched_config(n_sys=args.systems or 4096)
        batch = bm.BandedBatch(n, kl, ku, nrhs, torch.float64, dev)
        for s in range(batch.count):
            mb = batch.matrix_band(s)
            mb.normal_(generator=g)
            mb[int(ku[s])] += 2.0 * (kl[s] + ku[s])
            batch.rhs(s).normal_(generator=g)
        AB0, B0 = batch.AB.clone(), batch.B.clone()
        if parts[1] == "plain":
            def fn():
                batch.AB.copy_(AB0)
                batch.B.copy_(B0)
                batch.factor_solve()
        else:
            fn = lambda: batch.solve_mixed(1e-10, 30)
    elif parts[0] == "lu":
        n = args.n or 10000
        A = bm.BandedMatrix(bm.band_storage(2 * lu + 1, n, dt, dev), n, lu, lu)
        A.data.normal_(generator=g)
        A.data[lu] += 2.0 * lu + 1.0
        b = torch.randn(n, dtype=dt, device=dev, generator=g)
        fn = lambda: A.solve(b)
    elif parts[0] == "config1":
        # the CPU-runnable case: brandn(10000,10000,4,3) + 10 I, A\b
        n = args.n or 10000
        A = bm.brandn(torch.float64, n, n, 4, 3, device=dev, generator=g)
        A.data[3] += 10.0
        b = torch.randn(n, dtype=torch.float64, device=dev, generator=g)
        fn = lambda: A.solve(b)
    elif parts[0] == "refined":
        # the single-system refined solve (randn + 16 I, b randn), as refined_single times it
        n = args.n or (1 << 20)
        A = bm.BandedMatrix(bm.band_storage(2 * lu + 1, n, torch.float64, dev), n, lu, lu)
        A.data.normal_(generator=g)
        A.data[lu] += 16.0
        b = torch.randn(n, dtype=torch.float64, device=dev, generator=g)
        fn = lambda: bm.solve_refined(A, b, tol=1e-10)
    elif parts[0] == "qr":
        n = args.n or (1 << 18)
        A = bm.BandedMatrix(bm.band_storage(2 * lu + 1, n, dt, dev), n, lu, lu)
        A.data.normal_(generator=g)
        fn = lambda: bm.qr(A)
    else:
        raise SystemExit(f"unknown case {name}")
    fn()
    torch.cuda.synchronize()
    for r in range(args.reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        print(f"{name} rep {r}: {e0.elapsed_time(e1):.3f} ms", flush=True)
    del np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sweep-only", action="store_true", help="time only the gbmv/gbmm sweep")
    ap.add_argument("--case", default=None, help="run one named workload (profiler captures)")
    ap.add_argument("--n", type=int, default=0, help="--case: matrix order")
    ap.add_argument("--reps", type=int, default=3, help="--case: repetitions")
    ap.add_argument("--systems", type=int, default=0, help="--case batched_*: number of systems")
    args = ap.parse_args()
    if args.case:
        run_case(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        cb = cpu_sweep(args.steps, args.warmup)
        cpu = {"value": cb["value"], "unit": "GB/s", "cores": cb["threads"], "kind": "reference",
               "sample": cb["sample"], "host_cores": cb["host_cores"], "gbmv_GBps": cb["gbmv_GBps"],
               "gbmm_GBps": cb["gbmm_GBps"], "one_thread": cb.get("one_thread")}
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "GB/s", "n_gpus": args.gpus,
            "steps": cb["steps"], "warmup": cb["warmup"], "ms_per_step": cb["sec_per_step"] * 1e3,
            "timed_s": cb["sec_total"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64", "data": "synthetic (numpy PCG64, seeded)", "config": bench_config(args.gpus),
            "cpu_baseline": cpu,
            "e2e": {"value": cb["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }))
        return

    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    out = run_gpu(args, rank, world)
    if rank == 0 and not args.sweep_only:
        import torch

        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
        stream = torch.cuda.current_stream(dev)
        bm = __import__("__graft_entry__").package()
        out["batched_solve"] = run_batched(bm, dev, stream)
        bs = out["batched_solve"]
        # the metric's other half: systems/s of the 4096-system batch, plain FP64 against
        # the FP32-factor / FP64-refined solve at 1e-10 backward error
        out["systems_per_s"] = {"plain_fp64": bs["plain_fp64"]["systems_per_s"],
                                "refined_1e-10": bs["mixed_fp32_fp64_refined"]["systems_per_s"],
                                "refined_vs_plain": bs["speedup_mixed_vs_plain"],
                                "workload": bs["workload"]}
        torch.cuda.empty_cache()
        out["cpu_runnable"] = run_cpu_runnable(bm, dev, stream)
        out["qr_least_squares"] = run_qr(bm, dev, stream)
        torch.cuda.empty_cache()
        out["refined_single"] = run_refined(bm, dev, stream)
        torch.cuda.empty_cache()
        out["pde_adjoint"] = run_pde(bm, dev, stream)
    if rank == 0:
        if not args.no_cpu_baseline:
            if not args.sweep_only:
                out["cpu_baseline_solvers"] = cpu_lu_baselines()
            cb = cpu_sweep(5, 1, one_thread_steps=1)
            out["cpu_baseline"] = {"value": cb["value"], "unit": "GB/s", "cores": cb["threads"], "kind": "reference",
                                   "sample": cb["sample"], "host_cores": cb["host_cores"],
                                   "gbmv_GBps": cb["gbmv_GBps"], "gbmm_GBps": cb["gbmm_GBps"],
                                   "one_thread": cb.get("one_thread")}
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
