"""bandedgpu: BandedMatrices.jl's banded hot path (gbmv, banded*banded, banded LU and
QR, plus batched, mixed-precision and adjoint solves) on one GB300 GPU.

The numerical work runs in libbandedgpu.so (hand-written CUDA for sm_103a behind
the C ABI in include/bandedgpu.h).  This package is the host-side mirror of the
reference's Julia interface: a device-resident ``BandedMatrix`` that keeps the
(l+u+1) x n LAPACK band storage, ``brand``/``brandn``, ``mul_`` (``mul!``),
``@`` (``*``), ``lu``, ``ldiv_`` (``ldiv!``), ``solve`` (``\\``) and ``qr``.
"""
from . import _lib
from ._lib import BandedGPUError
from .banded import (BandedMatrix, BandError, DimensionMismatch, band_storage, bandeddata, bandwidth, bandwidths,
                     brand, brandn, gbmv)
from .gbmm import banded_mul, banded_mul_, gbmm, nonzero_bands, prodbandwidths
from .linalg import ldiv, mul, mul_, mul_t_
from .lu import BandedLU, ldiv_, lu, lu_, transpose
from .batched import BandedBatch, lpt_order
from .qr import BandedQR, lmul_, qr
from .autograd import BandedSolve, banded_solve
from .refine import solve_refined
from .tri import (LowerTriangular, UnitLowerTriangular, UnitUpperTriangular, UpperTriangular, dense_gbmm_,
                  gbmm_dense_)
from .symbanded import BandedCholesky, Symmetric, cholesky
from .elementwise import add, axpy_, dot, scale_, shift_
from .convert import from_rows, from_sparse, sparse, sparse_bandwidths
from . import pde, shard

__all__ = [
    "BandedGPUError", "BandedMatrix", "BandError", "DimensionMismatch", "band_storage", "bandeddata",
    "bandwidth", "bandwidths", "brand", "brandn", "gbmv", "ldiv", "mul", "mul_", "mul_t_", "load_library",
    "banded_mul", "banded_mul_", "gbmm", "nonzero_bands", "prodbandwidths",
    "BandedLU", "ldiv_", "lu", "lu_", "transpose", "BandedBatch", "lpt_order", "BandedQR", "lmul_", "qr",
    "solve_refined", "UpperTriangular", "LowerTriangular", "UnitUpperTriangular", "UnitLowerTriangular",
    "gbmm_dense_", "dense_gbmm_", "Symmetric", "BandedCholesky", "cholesky",
    "axpy_", "scale_", "shift_", "add", "dot", "sparse", "sparse_bandwidths", "from_sparse", "from_rows",
    "BandedSolve", "banded_solve",
]


def load_library():
    """Load libbandedgpu.so (raises if it has not been built)."""
    return _lib.load()
