"""Device-resident BandedMatrix: the storage contract and constructors of
BandedMatrices.jl (src/banded/BandedMatrix.jl) with its entries in GPU memory.

``A.data`` is a torch tensor of shape (l+u+1, n) whose memory is LAPACK band
storage, column-major with leading dimension ``A.lda`` (stride (1, lda)), so
``A[k, j] == A.data[u + k - j, j]`` (inbands_getindex,
src/banded/BandedMatrix.jl:414-419).  ``A.m`` is the number of rows (the
reference's ``raxis``).  Bandwidths may be negative, as in the reference.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib


class DimensionMismatch(ValueError):
    """Raised where Julia would throw DimensionMismatch."""


class BandError(ValueError):
    """Raised where BandedMatrices.jl throws BandError (src/generic/Band.jl:75-88)."""


_FLOATS = (torch.float64, torch.float32)


def _prefix(dtype: torch.dtype) -> str:
    if dtype == torch.float64:
        return "d"
    if dtype == torch.float32:
        return "s"
    raise TypeError(f"unsupported element type {dtype}: Float64 and Float32 are supported")


def _stream(device: torch.device) -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _scalar(dtype: torch.dtype, v: float):
    return ctypes.c_double(v) if dtype == torch.float64 else ctypes.c_float(v)


def _ptr(t: torch.Tensor, offset_elems: int = 0) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr() + offset_elems * t.element_size())


def _require_cuda(*ts: torch.Tensor) -> None:
    for t in ts:
        if not t.is_cuda:
            raise ValueError("bandedgpu operates on device-resident (CUDA) tensors only")


def band_storage(rows: int, n: int, dtype=torch.float64, device="cuda", lda: int | None = None,
                 fill: float | None = None) -> torch.Tensor:
    """A (rows x n) column-major tensor (stride (1, lda)), i.e. LAPACK band storage."""
    lda = max(1, lda or rows)
    buf = torch.empty((n, lda), dtype=dtype, device=device)
    if fill is not None:
        buf.fill_(fill)
    return buf.t()[:rows, :]


class BandedMatrix:
    """m x n banded matrix with bandwidths (l, u) and device band storage ``data``."""

    __slots__ = ("data", "m", "l", "u")

    def __init__(self, data: torch.Tensor, m: int, l: int, u: int):
        # _BandedMatrix(data, m, l, u): src/banded/BandedMatrix.jl:16-28
        if data.dim() != 2:
            raise ValueError("data must be a matrix")
        if data.shape[0] != l + u + 1 and not (data.shape[0] == 0 and -l > u):
            raise ValueError("Data matrix must have number rows equal to number of bands")
        if data.shape[1] > 1 and data.shape[0] > 1 and data.stride(0) != 1:
            raise ValueError("band storage must be column-major (stride(0) == 1)")
        self.data, self.m, self.l, self.u = data, int(m), int(l), int(u)

    # -- interface (src/generic/AbstractBandedMatrix.jl) ---------------------
    @property
    def n(self) -> int:
        return int(self.data.shape[1])

    @property
    def shape(self) -> tuple[int, int]:
        return (self.m, self.n)

    @property
    def dtype(self) -> torch.dtype:
        return self.data.dtype

    @property
    def device(self) -> torch.device:
        return self.data.device

    @property
    def lda(self) -> int:
        return max(1, int(self.data.stride(1))) if self.data.shape[1] > 1 else max(1, self.data.shape[0])

    def bandwidths(self) -> tuple[int, int]:
        return (self.l, self.u)

    def __repr__(self) -> str:
        return f"BandedMatrix({self.m}x{self.n}, bandwidths=({self.l},{self.u}), {self.dtype}, {self.device})"

    # -- constructors --------------------------------------------------------
    @staticmethod
    def undef(shape, bands, dtype=torch.float64, device="cuda") -> "BandedMatrix":
        """BandedMatrix{T}(undef, (m,n), (l,u)) (src/banded/BandedMatrix.jl:51-68)."""
        (m, n), (l, u) = shape, bands
        return BandedMatrix(band_storage(max(0, l + u + 1), n, dtype, device), m, l, u)

    @staticmethod
    def zeros(shape, bands, dtype=torch.float64, device="cuda") -> "BandedMatrix":
        (m, n), (l, u) = shape, bands
        return BandedMatrix(band_storage(max(0, l + u + 1), n, dtype, device, fill=0.0), m, l, u)

    @staticmethod
    def from_dense(A: torch.Tensor, bands) -> "BandedMatrix":
        """BandedMatrix(A, (l,u)) (src/banded/BandedMatrix.jl:222-232): copies the in-band
        entries of a dense matrix; the off-matrix corner slots are zero here."""
        l, u = bands
        m, n = A.shape
        B = BandedMatrix.zeros((m, n), (l, u), A.dtype, A.device)
        j = torch.arange(n, device=A.device)
        for r in range(l + u + 1):
            k = j + r - u
            ok = (k >= 0) & (k < m)
            B.data[r, ok] = A[k[ok], j[ok]]
        return B

    def copy(self) -> "BandedMatrix":
        d = band_storage(self.data.shape[0], self.n, self.dtype, self.device)
        d.copy_(self.data)
        return BandedMatrix(d, self.m, self.l, self.u)

    def to_dense(self) -> torch.Tensor:
        """Matrix(A): dense device copy (test/diagnostic helper, not a hot path)."""
        A = torch.zeros(self.m, self.n, dtype=self.dtype, device=self.device)
        j = torch.arange(self.n, device=self.device)
        for r in range(max(0, self.l + self.u + 1)):
            k = j + r - self.u
            ok = (k >= 0) & (k < self.m)
            A[k[ok], j[ok]] = self.data[r, ok]
        return A

    def rewiden(self, bands) -> "BandedMatrix":
        """BandedMatrix{T}(A, (l2,u2)) with l2 >= l, u2 >= u: extra bands zero."""
        l2, u2 = bands
        if l2 < self.l or u2 < self.u:
            raise BandError("new bandwidths must contain the old ones")
        d = band_storage(l2 + u2 + 1, self.n, self.dtype, self.device, fill=0.0)
        d[u2 - self.u: u2 - self.u + self.l + self.u + 1, :] = self.data
        return BandedMatrix(d, self.m, l2, u2)

    # -- scalar indexing (0-based k, j; the reference's A[k+1, j+1]) -----------
    def _checkbounds(self, k: int, j: int) -> None:
        if not (0 <= k < self.m and 0 <= j < self.n):
            raise IndexError(f"index ({k}, {j}) is out of bounds for a {self.m}x{self.n} BandedMatrix")

    def __getitem__(self, idx):
        """A[k, j]: the band entry data[u + k - j, j], zero outside the band
        (banded_getindex / inbands_getindex, src/banded/BandedMatrix.jl:414-442).  Reads
        one element from the device: a diagnostic, not a hot path."""
        k, j = (int(i) for i in idx)
        self._checkbounds(k, j)
        if -self.l <= j - k <= self.u:
            return self.data[self.u + k - j, j].item()
        return 0.0

    def __setitem__(self, idx, v) -> None:
        """A[k, j] = v: writes the band entry; outside the band only v == 0 is accepted
        and BandError is raised otherwise (banded_setindex!,
        src/banded/BandedMatrix.jl:627-643)."""
        k, j = (int(i) for i in idx)
        self._checkbounds(k, j)
        if -self.l <= j - k <= self.u:
            self.data[self.u + k - j, j] = v
        elif v != 0:
            raise BandError(f"cannot set band {j - k} of a BandedMatrix with bandwidths ({self.l}, {self.u})")

    # -- operators -----------------------------------------------------------
    def __matmul__(self, other):
        from . import linalg
        return linalg.mul(self, other)

    def __add__(self, other):
        from .elementwise import add
        return add(self, other, 1.0)

    def __sub__(self, other):
        from .elementwise import add
        return add(self, other, -1.0)

    def __neg__(self):
        from .elementwise import scale_
        return scale_(-1.0, self.copy())

    def __mul__(self, alpha):
        from .elementwise import scale_
        return scale_(float(alpha), self.copy())

    __rmul__ = __mul__

    def __rmatmul__(self, D):
        """D * A for a dense D (src/generic/matmul.jl:258-271)."""
        from .tri import _empty_colmajor, dense_gbmm_
        return dense_gbmm_(_empty_colmajor(D.shape[0], self.n, D), D, self, 1.0, 0.0)

    def solve(self, b):
        """A \\ b (materialize!(::Ldiv), src/banded/linalg.jl:5-9)."""
        from . import linalg
        return linalg.ldiv(self, b)


def bandwidths(A: BandedMatrix) -> tuple[int, int]:
    return A.bandwidths()


def bandwidth(A: BandedMatrix, k: int) -> int:
    return A.bandwidths()[k - 1]


def bandeddata(A: BandedMatrix) -> torch.Tensor:
    return A.data


def _rand_fill(rows: int, n: int, dtype, device, generator, normal: bool) -> torch.Tensor:
    d = band_storage(rows, n, dtype, device)
    if rows * n:
        if normal:
            d.normal_(generator=generator)
        else:
            d.uniform_(0.0, 1.0, generator=generator)
    return d


def brand(dtype, m: int, n: int, l: int, u: int, *, device="cuda", generator=None) -> BandedMatrix:
    """brand(T, m, n, l, u) (src/banded/BandedMatrix.jl:184-204): uniform [0,1) in every
    storage slot, the off-matrix corners included."""
    return BandedMatrix(_rand_fill(max(0, l + u + 1), n, dtype, device, generator, False), m, l, u)


def brandn(dtype, m: int, n: int, l: int, u: int, *, device="cuda", generator=None) -> BandedMatrix:
    """brandn(T, m, n, l, u): standard normal entries in every storage slot."""
    return BandedMatrix(_rand_fill(max(0, l + u + 1), n, dtype, device, generator, True), m, l, u)


def gbmv(trans: str, alpha: float, A: BandedMatrix, x: torch.Tensor, beta: float, y: torch.Tensor,
         *, kl: int | None = None, ku: int | None = None, m: int | None = None) -> torch.Tensor:
    """Raw xGBMV on A's storage (BLAS.gbmv!, src/blas.jl:16-28); kl/ku/m default to A's."""
    _require_cuda(A.data, x, y)
    p = _prefix(A.dtype)
    if x.dtype != A.dtype or y.dtype != A.dtype:
        raise TypeError("gbmv: element types of A, x and y must agree")
    m = A.m if m is None else m
    kl = A.l if kl is None else kl
    ku = A.u if ku is None else ku
    incx = x.stride(0) if x.numel() > 1 else 1
    incy = y.stride(0) if y.numel() > 1 else 1
    _lib.call(f"bm_{p}gbmv", trans.encode(), m, A.n, kl, ku, _scalar(A.dtype, alpha), _ptr(A.data),
              A.lda, _ptr(x), incx, _scalar(A.dtype, beta), _ptr(y), incy, _stream(A.device))
    return y
