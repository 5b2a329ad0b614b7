// Format conversion between band storage and other layouts, on the device.
//
//   gb2csc  -- sparse(A) (ext/BandedMatricesSparseArraysExt.jl:7-9): every in-matrix
//              slot of the band becomes a stored entry (explicit zeros kept), as
//              sparse(_banded_rowval, _banded_colval, _banded_nzval) builds it
//              (src/banded/BandedMatrix.jl:796-836): slots outside the matrix are
//              clamped to row 1 or m with value 0 and summed into that entry (a column
//              with no in-matrix slot keeps one structural zero there).
//   csc_bandwidths -- bandwidths(::SparseMatrixCSC) (the extension's :11-33): the extreme
//              diagonals of the nonzero values; -max(m,n) each when every stored value
//              is zero, (-40320, -40320) (bandwidths(Zeros)) when nothing is stored.
//   csc2gb  -- BandedMatrix(S, (l,u)): the band storage filled from S (entries outside
//              the band are counted, not stored).
//   rows2cols -- the BandedRows copy of _BandedMatrix(::BandedRows, A)
//              (src/banded/BandedMatrix.jl:267-284): row-major band data R (row i holds
//              A(i, i-l .. i+u) at R[i + (c - i + l) * ldr]) to column-major band storage.
// All are streams over the band storage (HBM-bound).  Indices are 0-based int64.
#include <climits>

#include "common.cuh"

namespace bm {

__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }

__device__ __forceinline__ i64 col_lo(i64 c, i64 u) { return max((i64)0, c - u); }
__device__ __forceinline__ i64 col_hi(i64 c, i64 m, i64 l) { return min(m - 1, c + l); }

// entries of column c in sparse(A): the in-matrix slots, or one clamped zero
__device__ __forceinline__ i64 csc_count(i64 c, i64 m, i64 l, i64 u) {
  if (l + u + 1 <= 0 || m == 0) return 0;
  const i64 k = col_hi(c, m, l) - col_lo(c, u) + 1;
  return k > 0 ? k : 1;
}

__global__ void csc_count_kernel(i64 m, i64 n, i64 l, i64 u, i64* colptr) {
  for (i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (i64)gridDim.x * blockDim.x)
    colptr[c + 1] = csc_count(c, m, l, u);
  if (blockIdx.x == 0 && threadIdx.x == 0) colptr[0] = 0;
}

// In-place inclusive scan of v[1..len] (v[0] == 0) by one CTA: each thread scans its own
// contiguous segment, the segment totals are scanned across the CTA, then each segment
// adds its offset.
constexpr int kScanThreads = 1024;
__global__ void __launch_bounds__(kScanThreads) scan_kernel(i64* v, i64 len) {
  __shared__ i64 tot[kScanThreads];
  const i64 seg = (len + kScanThreads - 1) / kScanThreads;
  const i64 b = 1 + threadIdx.x * seg, e = min(1 + len, b + seg);
  i64 s = 0;
  for (i64 i = b; i < e; ++i) s += v[i];
  tot[threadIdx.x] = s;
  __syncthreads();
  for (int w = 1; w < kScanThreads; w <<= 1) {
    const i64 x = threadIdx.x >= w ? tot[threadIdx.x - w] : 0;
    __syncthreads();
    tot[threadIdx.x] += x;
    __syncthreads();
  }
  i64 acc = threadIdx.x ? tot[threadIdx.x - 1] : 0;
  for (i64 i = b; i < e; ++i) {
    acc += v[i];
    v[i] = acc;
  }
}

template <typename T>
__global__ void gb2csc_fill_kernel(i64 m, i64 n, i64 l, i64 u, const T* __restrict__ A, i64 lda,
                                   const i64* __restrict__ colptr, i64* __restrict__ rowval, T* __restrict__ nzval) {
  const i64 rows = l + u + 1, tot = rows * n;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
    const i64 c = e / rows, r = e - c * rows;
    const i64 k = c + r - u, lo = col_lo(c, u), hi = col_hi(c, m, l);
    if (hi < lo) {  // no in-matrix slot: one clamped structural zero
      if (r == 0) {
        rowval[colptr[c]] = (c - u > m - 1) ? m - 1 : 0;
        nzval[colptr[c]] = T(0);
      }
      continue;
    }
    if (k < lo || k > hi) continue;
    T v = A[r + c * lda];
    // clamped out-of-matrix slots of this column are summed into rows 0 and m-1
    if ((k == 0 && c - u < 0) || (k == m - 1 && c + l > m - 1)) v = add_rn(v, T(0));
    const i64 p = colptr[c] + (k - lo);
    rowval[p] = k;
    nzval[p] = v;
  }
}

__global__ void bw_init_kernel(i64 m, i64 n, i64* lu) {
  lu[0] = lu[1] = -max(m, n);
}

template <typename T>
__global__ void csc_bw_kernel(i64 n, const i64* __restrict__ colptr, const i64* __restrict__ rowval,
                              const T* __restrict__ nzval, i64* lu) {
  i64 l = LLONG_MIN, u = LLONG_MIN;
  for (i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (i64)gridDim.x * blockDim.x)
    for (i64 p = colptr[c]; p < colptr[c + 1]; ++p) {
      if (nzval[p] == T(0)) continue;  // explicit zeros do not count
      const i64 i = rowval[p];
      u = max(u, c - i);
      l = max(l, i - c);
    }
  if (l != LLONG_MIN) atomicMax(reinterpret_cast<long long*>(lu), (long long)l);
  if (u != LLONG_MIN) atomicMax(reinterpret_cast<long long*>(lu + 1), (long long)u);
}

__global__ void bw_empty_kernel(i64 n, const i64* colptr, i64* lu) {
  if (colptr[n] == 0) lu[0] = lu[1] = -40320;
}

template <typename T>
__global__ void fill_zero_kernel(i64 rows, i64 n, T* A, i64 lda) {
  const i64 tot = rows * n;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
    const i64 c = e / rows, r = e - c * rows;
    A[r + c * lda] = T(0);
  }
}

template <typename T>
__global__ void csc2gb_kernel(i64 m, i64 n, i64 l, i64 u, const i64* __restrict__ colptr,
                              const i64* __restrict__ rowval, const T* __restrict__ nzval, T* __restrict__ A, i64 lda,
                              unsigned long long* dropped) {
  unsigned long long drop = 0;
  for (i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (i64)gridDim.x * blockDim.x)
    for (i64 p = colptr[c]; p < colptr[c + 1]; ++p) {
      const i64 i = rowval[p], d = i - c;
      if (i < 0 || i >= m || d > l || d < -u) {
        drop += nzval[p] != T(0);
        continue;
      }
      A[(u + d) + c * lda] = nzval[p];
    }
  if (drop) atomicAdd(dropped, drop);
}

template <typename T>
__global__ void rows2cols_kernel(i64 m, i64 n, i64 l, i64 u, const T* __restrict__ R, i64 ldr, T* __restrict__ A,
                                 i64 lda) {
  const i64 rows = l + u + 1, tot = rows * n;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
    const i64 c = e / rows, r = e - c * rows;
    const i64 i = c + r - u;  // A(i, c) at storage row r
    if (i >= 0 && i < m) A[r + c * lda] = R[i + (c - i + l) * ldr];
  }
}

static unsigned grid_of(i64 tot) {
  return (unsigned)std::max<i64>(1, std::min<i64>(ceil_div(tot, 256), (i64)num_sms() * 16));
}

template <typename T>
static int gb2csc_impl(i64 m, i64 n, i64 l, i64 u, const T* A, i64 lda, i64* colptr, i64* rowval, T* nzval,
                       cudaStream_t s, const char* name) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (l + u + 1 > 0 && lda < l + u + 1) return -6;
  if (!colptr) return -7;
  csc_count_kernel<<<grid_of(std::max<i64>(n, 1)), 256, 0, s>>>(m, n, l, u, colptr);
  int r = launch_status(name);
  if (r) return r;
  scan_kernel<<<1, kScanThreads, 0, s>>>(colptr, n);
  if ((r = launch_status(name))) return r;
  if (n == 0 || m == 0 || l + u + 1 <= 0) return BM_OK;
  gb2csc_fill_kernel<T><<<grid_of((l + u + 1) * n), 256, 0, s>>>(m, n, l, u, A, lda, colptr, rowval, nzval);
  return launch_status(name);
}

template <typename T>
static int csc_bandwidths_impl(i64 m, i64 n, const i64* colptr, const i64* rowval, const T* nzval, i64* lu,
                               cudaStream_t s, const char* name) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (!colptr) return -3;
  if (!lu) return -6;
  bw_init_kernel<<<1, 1, 0, s>>>(m, n, lu);
  int r = launch_status(name);
  if (r) return r;
  if (n > 0) {
    csc_bw_kernel<T><<<grid_of(n), 256, 0, s>>>(n, colptr, rowval, nzval, lu);
    if ((r = launch_status(name))) return r;
  }
  bw_empty_kernel<<<1, 1, 0, s>>>(n, colptr, lu);
  return launch_status(name);
}

template <typename T>
static int csc2gb_impl(i64 m, i64 n, const i64* colptr, const i64* rowval, const T* nzval, i64 l, i64 u, T* A,
                       i64 lda, unsigned long long* dropped, cudaStream_t s, const char* name) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (!colptr) return -3;
  if (l + u + 1 > 0 && lda < l + u + 1) return -9;
  if (!dropped) return -10;
  int r = cuda_status(cudaMemsetAsync(dropped, 0, sizeof(unsigned long long), s), name);
  if (r || n == 0 || l + u + 1 <= 0) return r;
  fill_zero_kernel<T><<<grid_of((l + u + 1) * n), 256, 0, s>>>(l + u + 1, n, A, lda);
  if ((r = launch_status(name))) return r;
  csc2gb_kernel<T><<<grid_of(n), 256, 0, s>>>(m, n, l, u, colptr, rowval, nzval, A, lda, dropped);
  return launch_status(name);
}

template <typename T>
static int rows2cols_impl(i64 m, i64 n, i64 l, i64 u, const T* R, i64 ldr, T* A, i64 lda, cudaStream_t s,
                          const char* name) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (l + u + 1 <= 0) return BM_OK;
  if (ldr < std::max<i64>(1, m)) return -6;
  if (lda < l + u + 1) return -8;
  if (m == 0 || n == 0) return BM_OK;
  rows2cols_kernel<T><<<grid_of((l + u + 1) * n), 256, 0, s>>>(m, n, l, u, R, ldr, A, lda);
  return launch_status(name);
}

}  // namespace bm

#define BM_CONVERT(P, T)                                                                                            \
  extern "C" int bm_##P##gb2csc(int64_t m, int64_t n, int64_t l, int64_t u, const T* A, int64_t lda,               \
                                int64_t* colptr, int64_t* rowval, T* nzval, bm_stream_t stream) {                   \
    return bm::gb2csc_impl<T>(m, n, l, u, A, lda, colptr, rowval, nzval, reinterpret_cast<cudaStream_t>(stream),    \
                              "bm_" #P "gb2csc");                                                                   \
  }                                                                                                                 \
  extern "C" int bm_##P##csc_bandwidths(int64_t m, int64_t n, const int64_t* colptr, const int64_t* rowval,        \
                                        const T* nzval, int64_t* lu, bm_stream_t stream) {                          \
    return bm::csc_bandwidths_impl<T>(m, n, colptr, rowval, nzval, lu, reinterpret_cast<cudaStream_t>(stream),      \
                                      "bm_" #P "csc_bandwidths");                                                   \
  }                                                                                                                 \
  extern "C" int bm_##P##csc2gb(int64_t m, int64_t n, const int64_t* colptr, const int64_t* rowval, const T* nzval, \
                                int64_t l, int64_t u, T* A, int64_t lda, unsigned long long* dropped,                \
                                bm_stream_t stream) {                                                               \
    return bm::csc2gb_impl<T>(m, n, colptr, rowval, nzval, l, u, A, lda, dropped,                                   \
                              reinterpret_cast<cudaStream_t>(stream), "bm_" #P "csc2gb");                           \
  }                                                                                                                 \
  extern "C" int bm_##P##gbrows2cols(int64_t m, int64_t n, int64_t l, int64_t u, const T* R, int64_t ldr, T* A,    \
                                     int64_t lda, bm_stream_t stream) {                                             \
    return bm::rows2cols_impl<T>(m, n, l, u, R, ldr, A, lda, reinterpret_cast<cudaStream_t>(stream),                \
                                 "bm_" #P "gbrows2cols");                                                           \
  }

BM_CONVERT(d, double)
BM_CONVERT(s, float)

// Number of stored entries sparse(A) has for an m x n band (l, u): a host-side count
// (every in-matrix band slot, plus one structural zero per column without one).
extern "C" int64_t bm_gb2csc_nnz(int64_t m, int64_t n, int64_t l, int64_t u) {
  if (m <= 0 || n <= 0 || l + u + 1 <= 0) return 0;
  int64_t nnz = 0;
  for (int64_t c = 0; c < n; ++c) {
    const int64_t lo = std::max<int64_t>(0, c - u), hi = std::min<int64_t>(m - 1, c + l);
    nnz += hi >= lo ? hi - lo + 1 : 1;
  }
  return nnz;
}
