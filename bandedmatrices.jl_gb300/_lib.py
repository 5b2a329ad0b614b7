"""ctypes binding of libbandedgpu.so (the C ABI declared in include/bandedgpu.h).

This is the Python counterpart of the ``ccall`` bindings a Julia package would
make.  There is no fallback: if the shared library is missing or no CUDA device
is present, every call raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libbandedgpu.so")

BM_OK = 0
BM_ERR_CUDA = -1001
BM_ERR_UNSUPPORTED = -1002
BM_ERR_NOMEM = -1003
BM_ERR_ALIGN = -1004

i64 = ctypes.c_int64
P = ctypes.c_void_p
D = ctypes.c_double
F = ctypes.c_float
C = ctypes.c_char
I = ctypes.c_int

# name -> argtypes (every entry point returns int, except bm_last_error and bm_launch_count)
SIGNATURES: dict[str, list] = {
    "bm_version": [],
    "bm_last_error": [],
    "bm_device_status": [P, I, P],
    "bm_launch_count": [],
    "bm_probe_fma_rate": [I, P, P],
    "bm_wait_selftest": [i64, P, P],
    "bm_dgbmv": [C, i64, i64, i64, i64, D, P, i64, P, i64, D, P, i64, P],
    "bm_sgbmv": [C, i64, i64, i64, i64, F, P, i64, P, i64, F, P, i64, P],
    "bm_dgbmm": [i64] * 9 + [D, P, i64, P, i64, D, P, i64, P],
    "bm_sgbmm": [i64] * 9 + [F, P, i64, P, i64, F, P, i64, P],
    "bm_dgb_nonzero_bands": [i64, i64, i64, i64, P, i64, P, P],
    "bm_sgb_nonzero_bands": [i64, i64, i64, i64, P, i64, P, P],
    "bm_dgbtrf": [i64, i64, i64, i64, P, i64, P, P, P],
    "bm_sgbtrf": [i64, i64, i64, i64, P, i64, P, P, P],
    "bm_dgbtrs": [C, i64, i64, i64, i64, P, i64, P, P, i64, P],
    "bm_sgbtrs": [C, i64, i64, i64, i64, P, i64, P, P, i64, P],
    "bm_dgbsv_batched": [i64, P, P, P, P, P, P, P, i64, i64, P],
    "bm_sgbsv_batched": [i64, P, P, P, P, P, P, P, i64, i64, P],
    "bm_dgbsv_batched_noalloc": [i64, P, P, P, P, P, i64, i64, P],
    "bm_dgbqrf": [i64, i64, i64, i64, P, i64, P, P],
    "bm_sgbqrf": [i64, i64, i64, i64, P, i64, P, P],
    "bm_dgbqr_lmul": [C, i64, i64, i64, i64, P, i64, P, i64, i64, P, i64, P],
    "bm_sgbqr_lmul": [C, i64, i64, i64, i64, P, i64, P, i64, i64, P, i64, P],
    "bm_dtbsv": [C, C, C, i64, i64, P, i64, P, i64, P],
    "bm_stbsv": [C, C, C, i64, i64, P, i64, P, i64, P],
    "bm_dtbmv": [C, C, C, i64, i64, P, i64, P, i64, P],
    "bm_stbmv": [C, C, C, i64, i64, P, i64, P, i64, P],
    "bm_dpbtrf": [C, i64, i64, P, i64, P, P],
    "bm_spbtrf": [C, i64, i64, P, i64, P, P],
    "bm_dpbtrs": [C, i64, i64, i64, P, i64, P, i64, P],
    "bm_spbtrs": [C, i64, i64, i64, P, i64, P, i64, P],
    "bm_dsbmv": [C, i64, i64, D, P, i64, P, i64, D, P, i64, P],
    "bm_ssbmv": [C, i64, i64, F, P, i64, P, i64, F, P, i64, P],
    "bm_dgbaxpy": [i64, i64, D, i64, i64, P, i64, i64, i64, P, i64, P, P],
    "bm_sgbaxpy": [i64, i64, F, i64, i64, P, i64, i64, i64, P, i64, P, P],
    "bm_dgbscal": [i64, i64, i64, i64, D, P, i64, P],
    "bm_sgbscal": [i64, i64, i64, i64, F, P, i64, P],
    "bm_dgbshift": [i64, i64, i64, i64, D, P, i64, P],
    "bm_sgbshift": [i64, i64, i64, i64, F, P, i64, P],
    "bm_dgbdot": [i64, i64, i64, i64, P, P, i64, P, P, P, P],
    "bm_sgbdot": [i64, i64, i64, i64, P, P, i64, P, P, P, P],
    "bm_plan_create": [P, i64, P, P, I, P, P, P],
    "bm_plan_destroy": [P],
    "bm_plan_schedule": [P, P, P, P],
    "bm_plan_execute_dgbsv": [P, P, P, P, P, P, P],
    "bm_plan_execute_dsgbsv": [P, P, P, P, P, P, P, P, P, P, P, D, i64, P],
    "bm_gb2csc_nnz": [i64, i64, i64, i64],
    "bm_dgb2csc": [i64, i64, i64, i64, P, i64, P, P, P, P],
    "bm_sgb2csc": [i64, i64, i64, i64, P, i64, P, P, P, P],
    "bm_dcsc_bandwidths": [i64, i64, P, P, P, P, P],
    "bm_scsc_bandwidths": [i64, i64, P, P, P, P, P],
    "bm_dcsc2gb": [i64, i64, P, P, P, i64, i64, P, i64, P, P],
    "bm_scsc2gb": [i64, i64, P, P, P, i64, i64, P, i64, P, P],
    "bm_dgbrows2cols": [i64, i64, i64, i64, P, i64, P, i64, P],
    "bm_sgbrows2cols": [i64, i64, i64, i64, P, i64, P, i64, P],
    "bm_dgbmm_bd": [i64] * 5 + [D, P, i64, P, i64, D, P, i64, P],
    "bm_sgbmm_bd": [i64] * 5 + [F, P, i64, P, i64, F, P, i64, P],
    "bm_dgbmm_db": [i64] * 5 + [D, P, i64, P, i64, D, P, i64, P],
    "bm_sgbmm_db": [i64] * 5 + [F, P, i64, P, i64, F, P, i64, P],
    "bm_dgbsv_adjoint": [i64, i64, i64, i64, P, i64, P, P, P, P, P, P, i64, P, P],
    "bm_sgbsv_adjoint": [i64, i64, i64, i64, P, i64, P, P, P, P, P, P, i64, P, P],
    "bm_dsgbsv_batched": [i64, P, P, P, P, P, P, P, P, P, P, P, P, D, i64, i64, i64, P],
    "bm_dgbsv_batched_sched": [i64, P, P, P, P, P, P, P, P, P],
    "bm_sgbsv_batched_sched": [i64, P, P, P, P, P, P, P, P, P],
    "bm_dsgbsv_batched_sched": [i64, P, P, P, P, P, P, P, P, P, P, P, P, P, D, i64, P],
    "bm_dsgbsv": [i64, i64, i64, i64, P, i64, P, i64, P, i64, P, P, P, D, i64, P, P, P, P],
    "bm_sgbtrf_tc": [i64, i64, i64, P, i64, P, i64, P, P, P],
}

# bm_gb_desc as a numpy structured dtype (9 x int64, C layout)
DESC_FIELDS = ["n", "kl", "ku", "nrhs", "ab_offset", "ldab", "b_offset", "ldb", "ipiv_offset"]


class BandedGPUError(RuntimeError):
    """A libbandedgpu call failed (illegal argument or CUDA error)."""


_lib = None


def load(path: str | None = None) -> ctypes.CDLL:
    """Load the shared library (once) and declare every signature."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise BandedGPUError(
            f"{path} is missing: build it with __graft_entry__.build() (there is no CPU fallback)")
    L = ctypes.CDLL(path)
    for name, argt in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = argt
        fn.restype = (ctypes.c_char_p if name == "bm_last_error"
                      else ctypes.c_ulonglong if name == "bm_launch_count"
                      else ctypes.c_int64 if name == "bm_gb2csc_nnz" else ctypes.c_int)
    _lib = L
    return L


def check(ret: int, name: str) -> None:
    if ret == BM_OK:
        return
    L = load()
    msg = L.bm_last_error().decode(errors="replace")
    if ret < 0 and ret > -100:
        raise BandedGPUError(f"{name}: illegal value of argument {-ret}")
    raise BandedGPUError(f"{name}: error {ret}: {msg}")


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)
