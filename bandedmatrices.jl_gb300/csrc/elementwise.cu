// Banded elementwise algebra: Y <- a X + Y (banded_axpy!), A <- alpha A (banded_lmul!),
// the diagonal shift A + sigma I, and the bilinear form dot(x, A, y).
//
// Replaces banded_axpy! / banded_generic_axpy! (src/banded/BandedMatrix.jl:1006-1015,
// src/generic/broadcast.jl:978-1020), banded_lmul! (src/generic/broadcast.jl:960-965)
// and _dot (src/banded/dot.jl:1-22).  These are HBM-bound streams over band storage.
//
//   axpy, equal bandwidths: axpy!(a, X.data, Y.data) in the reference, i.e. BLAS daxpy
//     over the whole storage: y <- fma(a, x, y) element for element.
//   axpy, different bandwidths: first every stored in-matrix entry of X outside Y's bands
//     must be zero (else BandError for the first such (k, j) in column order, reported
//     as the device index j*m + k and Y left untouched); then the overlapping bands get
//     y <- a*x + y, rounded twice as Julia evaluates it (no contraction).
//   dot(x, A, y) = sum_j y_j (sum_i A(i,j) x_i): column sums in ascending i, columns
//     with y_j == 0 skipped; the sum over columns is a fixed two-level tree (per-block
//     partials, then one block), so the result is deterministic.  The reference's @simd
//     loop leaves its summation order to the compiler, so results agree to rounding.
#include "common.cuh"

namespace bm {

// a * x rounded once, never contracted into a following add
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }

template <typename T>
__global__ void axpy_storage_kernel(i64 rows, i64 n, T a, const T* __restrict__ X, i64 ldx, T* __restrict__ Y,
                                    i64 ldy) {
  const i64 tot = rows * n;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
    const i64 j = e / rows, r = e - j * rows;
    Y[r + j * ldy] = fma(a, X[r + j * ldx], Y[r + j * ldy]);
  }
}

// bad <- min over nonzero in-matrix X(k, j) outside Y's bands of j*m + k
template <typename T>
__global__ void axpy_check_kernel(i64 m, i64 n, i64 Xl, i64 Xu, const T* __restrict__ X, i64 ldx, i64 Yl, i64 Yu,
                                  unsigned long long* bad) {
  const i64 rows = Xl + Xu + 1, tot = rows * n;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
    const i64 j = e / rows, r = e - j * rows;
    const i64 k = j + r - Xu, d = k - j;
    if (k < 0 || k >= m || (d <= Yl && d >= -Yu)) continue;
    if (X[r + j * ldx] != T(0)) atomicMin(bad, (unsigned long long)(j * m + k));
  }
}

template <typename T>
__global__ void axpy_bands_kernel(i64 m, i64 n, T a, i64 Xl, i64 Xu, const T* __restrict__ X, i64 ldx, i64 Yl,
                                  i64 Yu, T* __restrict__ Y, i64 ldy, const unsigned long long* bad) {
  if (*reinterpret_cast<volatile const unsigned long long*>(bad) != ~0ull) return;
  const i64 l = min(Xl, Yl), u = min(Xu, Yu), rows = l + u + 1, tot = rows * n;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
    const i64 j = e / rows, r = e - j * rows;
    const i64 k = j + r - u;
    if (k < 0 || k >= m) continue;
    T* yp = Y + (Yu + k - j) + j * ldy;
    *yp = mul_rn(a, X[(Xu + k - j) + j * ldx]) + *yp;  // two roundings, as Julia's a*x + y
  }
}

template <typename T>
__global__ void scal_storage_kernel(i64 rows, i64 n, T alpha, T* __restrict__ A, i64 lda) {
  const i64 tot = rows * n;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
    const i64 j = e / rows, r = e - j * rows;
    A[r + j * lda] = alpha * A[r + j * lda];
  }
}

template <typename T>
__global__ void shift_diag_kernel(i64 m, i64 n, i64 u, T sigma, T* __restrict__ A, i64 lda) {
  const i64 len = min(m, n);
  for (i64 j = (i64)blockIdx.x * blockDim.x + threadIdx.x; j < len; j += (i64)gridDim.x * blockDim.x)
    A[u + j * lda] += sigma;
}

constexpr int kDotThreads = 256;
constexpr int kDotBlocks = 1024;  // partial sums: the workspace the entry point asks for

template <typename T>
__global__ void __launch_bounds__(kDotThreads) dot_partial_kernel(i64 m, i64 n, i64 l, i64 u, const T* __restrict__ x,
                                                                  const T* __restrict__ A, i64 lda,
                                                                  const T* __restrict__ y, T* __restrict__ part) {
  __shared__ T red[kDotThreads];
  T s = T(0);
  for (i64 j = (i64)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (i64)gridDim.x * blockDim.x) {
    const T yj = y[j];
    if (yj == T(0)) continue;
    T t = T(0);
    const i64 i0 = max((i64)0, j - u), i1 = min(m - 1, j + l);
    for (i64 i = i0; i <= i1; ++i) t = fma(A[(u + i - j) + j * lda], x[i], t);
    s = fma(t, yj, s);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = kDotThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

template <typename T>
__global__ void __launch_bounds__(kDotThreads) dot_final_kernel(int nb, const T* __restrict__ part, T* out) {
  __shared__ T red[kDotThreads];
  T s = T(0);
  for (int b = threadIdx.x; b < nb; b += kDotThreads) s += part[b];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = kDotThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

static unsigned grid_for(i64 tot) { return (unsigned)std::max<i64>(1, std::min<i64>(ceil_div(tot, 256), (i64)num_sms() * 16)); }

template <typename T>
static int gbaxpy_impl(i64 m, i64 n, T a, i64 Xl, i64 Xu, const T* X, i64 ldx, i64 Yl, i64 Yu, T* Y, i64 ldy,
                       unsigned long long* bad, cudaStream_t s, const char* name) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (Xl + Xu + 1 > 0 && ldx < Xl + Xu + 1) return -7;
  if (Yl + Yu + 1 > 0 && ldy < Yl + Yu + 1) return -11;
  if (!bad) return -12;
  int r = cuda_status(cudaMemsetAsync(bad, 0xff, sizeof(unsigned long long), s), name);  // ~0: no violation
  if (r || m == 0 || n == 0 || -Xl > Xu) return r;
  if (Xl == Yl && Xu == Yu) {  // axpy!(a, X.data, Y.data)
    axpy_storage_kernel<T><<<grid_for((Xl + Xu + 1) * n), 256, 0, s>>>(Xl + Xu + 1, n, a, X, ldx, Y, ldy);
    return launch_status(name);
  }
  if (Xl > Yl || Xu > Yu) {
    axpy_check_kernel<T><<<grid_for((Xl + Xu + 1) * n), 256, 0, s>>>(m, n, Xl, Xu, X, ldx, Yl, Yu, bad);
    if ((r = launch_status(name))) return r;
  }
  if (-Yl > Yu || std::min(Xl, Yl) + std::min(Xu, Yu) + 1 <= 0) return BM_OK;
  axpy_bands_kernel<T><<<grid_for((std::min(Xl, Yl) + std::min(Xu, Yu) + 1) * n), 256, 0, s>>>(m, n, a, Xl, Xu, X, ldx,
                                                                                                Yl, Yu, Y, ldy, bad);
  return launch_status(name);
}

template <typename T>
static int gbscal_impl(i64 m, i64 n, i64 l, i64 u, T alpha, T* A, i64 lda, cudaStream_t s, const char* name) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (l + u + 1 > 0 && lda < l + u + 1) return -7;
  if (m == 0 || n == 0 || l + u + 1 <= 0) return BM_OK;
  scal_storage_kernel<T><<<grid_for((l + u + 1) * n), 256, 0, s>>>(l + u + 1, n, alpha, A, lda);
  return launch_status(name);
}

template <typename T>
static int gbshift_impl(i64 m, i64 n, i64 l, i64 u, T sigma, T* A, i64 lda, cudaStream_t s, const char* name) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (l < 0) return -3;
  if (u < 0) return -4;
  if (lda < l + u + 1) return -7;
  if (m == 0 || n == 0) return BM_OK;
  shift_diag_kernel<T><<<grid_for(std::min(m, n)), 256, 0, s>>>(m, n, u, sigma, A, lda);
  return launch_status(name);
}

template <typename T>
static int gbdot_impl(i64 m, i64 n, i64 l, i64 u, const T* x, const T* A, i64 lda, const T* y, T* result, T* work,
                      cudaStream_t s, const char* name) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (l < 0) return -3;
  if (u < 0) return -4;
  if (lda < l + u + 1) return -7;
  if (!result) return -9;
  if (!work) return -10;
  if (m == 0 || n == 0) return cuda_status(cudaMemsetAsync(result, 0, sizeof(T), s), name);
  const int nb = (int)std::min<i64>(kDotBlocks, ceil_div(n, (i64)kDotThreads));
  dot_partial_kernel<T><<<nb, kDotThreads, 0, s>>>(m, n, l, u, x, A, lda, y, work);
  int r = launch_status(name);
  if (r) return r;
  dot_final_kernel<T><<<1, kDotThreads, 0, s>>>(nb, work, result);
  return launch_status(name);
}

}  // namespace bm

#define BM_ELEMENTWISE(P, T)                                                                                         \
  extern "C" int bm_##P##gbaxpy(int64_t m, int64_t n, T a, int64_t Xl, int64_t Xu, const T* X, int64_t ldx,        \
                                int64_t Yl, int64_t Yu, T* Y, int64_t ldy, unsigned long long* bad,                 \
                                bm_stream_t stream) {                                                                \
    return bm::gbaxpy_impl<T>(m, n, a, Xl, Xu, X, ldx, Yl, Yu, Y, ldy, bad, reinterpret_cast<cudaStream_t>(stream), \
                              "bm_" #P "gbaxpy");                                                                    \
  }                                                                                                                  \
  extern "C" int bm_##P##gbscal(int64_t m, int64_t n, int64_t l, int64_t u, T alpha, T* A, int64_t lda,            \
                                bm_stream_t stream) {                                                                \
    return bm::gbscal_impl<T>(m, n, l, u, alpha, A, lda, reinterpret_cast<cudaStream_t>(stream), "bm_" #P "gbscal"); \
  }                                                                                                                  \
  extern "C" int bm_##P##gbshift(int64_t m, int64_t n, int64_t l, int64_t u, T sigma, T* A, int64_t lda,           \
                                 bm_stream_t stream) {                                                               \
    return bm::gbshift_impl<T>(m, n, l, u, sigma, A, lda, reinterpret_cast<cudaStream_t>(stream),                    \
                               "bm_" #P "gbshift");                                                                  \
  }                                                                                                                  \
  extern "C" int bm_##P##gbdot(int64_t m, int64_t n, int64_t l, int64_t u, const T* x, const T* A, int64_t lda,     \
                               const T* y, T* result, T* work, bm_stream_t stream) {                                 \
    return bm::gbdot_impl<T>(m, n, l, u, x, A, lda, y, result, work, reinterpret_cast<cudaStream_t>(stream),         \
                             "bm_" #P "gbdot");                                                                      \
  }

BM_ELEMENTWISE(d, double)
BM_ELEMENTWISE(s, float)
