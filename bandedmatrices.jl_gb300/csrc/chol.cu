// Symmetric positive definite band: Cholesky factorization (xPBTRF), its solve
// (xPBTRS) and the symmetric band product (xSBMV).
//
// Replaces pbtrf!/pbtrs! (src/lapack.jl:268-332), reached from banded_chol!
// (src/symbanded/BandedCholesky.jl:2-12, cholesky(Symmetric(A))), and sbmv!
// (src/blas.jl:35-64, Symmetric(A) * x).
//
// pbtrf follows LAPACK's unblocked xPBTF2 element by element: at step j the pivot
// a(j,j) must be > 0 (else info = j+1 and the factorization stops), its square root is
// stored, the kn = min(kd, n-1-j) entries of row j (upper) or column j (lower) are
// scaled by its reciprocal, and the trailing kn x kn triangle takes dsyr's rank-1
// update, each element once: a <- fma(x_s, -x_t, a) with the skip dsyr applies to a zero
// x.  One CTA keeps the (kd+1) x (kd+1) active triangle in shared memory as a ring in
// both dimensions (it slides one row and one column per step, the entering column read
// from the band); the update is spread over a 16 x 16 thread grid.  Factors therefore
// equal the oracle's bit for bit; OpenBLAS's blocked dpbtrf (kd >= 32) agrees to
// rounding.
//
// pbtrs is dpbtrs: two triangular band sweeps (tri.cu) per right-hand side.
// sbmv computes every output in reference DSBMV's order, one thread per output.
#include "tri.cuh"

namespace bm {

constexpr int kPbThreads = 256;

// The active triangle, oriented as the upper factor: element (s, t), s <= t (matrix row /
// column indices), lives at win[(t % W) * W + s % W].  For uplo = 'L' it holds L(t, s).
template <typename T, bool UPPER>
__global__ void __launch_bounds__(kPbThreads) pbtrf_kernel(i64 n, int kd, T* __restrict__ AB, i64 ldab, i64* info) {
  extern __shared__ __align__(16) unsigned char smem[];
  T* win = reinterpret_cast<T*>(smem);
  __shared__ int stop;
  const int tid = threadIdx.x, W = kd + 1;
  auto g = [&](i64 s, i64 t) -> i64 { return UPPER ? (kd + s - t) + t * ldab : (t - s) + s * ldab; };
  auto w = [&](i64 s, i64 t) -> T& { return win[(int)(t % W) * W + (int)(s % W)]; };
  for (int e = tid; e < W * W; e += kPbThreads) {
    const int t = e / W, s = e - t * W;
    if (s <= t && t < n) win[t * W + s] = AB[g(s, t)];
  }
  if (tid == 0) {
    stop = 0;
    *info = 0;
  }
  __syncthreads();
  const int ts = tid & 15, tt = tid >> 4;
  for (i64 j = 0; j < n; ++j) {
    const int kn = (int)min((i64)kd, n - 1 - j);
    if (tid == 0) {
      T ajj = w(j, j);
      if (!(ajj > T(0))) {
        *info = j + 1;
        stop = 1;
      } else {
        ajj = sqrt(ajj);
        w(j, j) = ajj;
        AB[g(j, j)] = ajj;
      }
    }
    __syncthreads();
    if (stop) break;
    const T r = T(1) / w(j, j);
    for (int t = 1 + tid; t <= kn; t += kPbThreads) {
      const T v = r * w(j, j + t);
      w(j, j + t) = v;
      AB[g(j, j + t)] = v;
    }
    __syncthreads();
    // rank-1 update of the trailing triangle (offsets 1 <= s <= t <= kn from j)
    for (int t = 1 + tt; t <= kn; t += 16) {
      const T xt = w(j, j + t);
      for (int s = 1 + ts; s <= t; s += 16) {
        const T xs = w(j, j + s);
        T& a = w(j + s, j + t);
        if (UPPER) {
          if (xt != T(0)) a = fma(xs, -xt, a);
        } else {  // dsyr 'L': element L(j+t, j+s) gets x_t * (-x_s), skipped when x_s == 0
          if (xs != T(0)) a = fma(xt, -xs, a);
        }
      }
    }
    __syncthreads();
    // slide: column j + W enters the slot column j leaves (rows j+1 .. j+W)
    if (j + W < n)
      for (int s = tid; s < W; s += kPbThreads) w(j + 1 + s, j + W) = AB[g(j + 1 + s, j + W)];
    __syncthreads();
  }
}

// y <- alpha A x + beta y for the symmetric band A (k off-diagonals), one thread per
// output, in reference DSBMV's order (see the oracle restatement): upper -- beta y_i,
// then column i (the diagonal term and alpha * the column's dot with x above the
// diagonal), then the columns i+1 .. i+k; lower -- beta y_i, the columns i-k .. i-1,
// then column i (diagonal term, then alpha * the dot below the diagonal).
template <typename T>
__global__ void sbmv_kernel(bool upper, i64 n, int k, T alpha, const T* __restrict__ A, i64 lda,
                            const T* __restrict__ x, i64 incx, T beta, T* __restrict__ y, i64 incy) {
  const i64 kx = incx > 0 ? 0 : -(n - 1) * incx, ky = incy > 0 ? 0 : -(n - 1) * incy;
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    T* yp = y + ky + i * incy;
    T acc = (beta == T(0)) ? T(0) : (beta == T(1) ? *yp : beta * *yp);
    if (alpha != T(0)) {
      if (upper) {
        T t2 = T(0);
        for (i64 r = max((i64)0, i - k); r < i; ++r) t2 = fma(A[(k - i + r) + i * lda], x[kx + r * incx], t2);
        acc = fma(alpha * x[kx + i * incx], A[k + i * lda], acc);
        acc = fma(alpha, t2, acc);
        const i64 hi = min(n - 1, i + k);
        for (i64 j = i + 1; j <= hi; ++j) acc = fma(alpha * x[kx + j * incx], A[(k - j + i) + j * lda], acc);
      } else {
        for (i64 j = max((i64)0, i - k); j < i; ++j) acc = fma(alpha * x[kx + j * incx], A[(i - j) + j * lda], acc);
        acc = fma(alpha * x[kx + i * incx], A[i * lda], acc);
        T t2 = T(0);
        const i64 hi = min(n - 1, i + k);
        for (i64 r = i + 1; r <= hi; ++r) t2 = fma(A[(r - i) + i * lda], x[kx + r * incx], t2);
        acc = fma(alpha, t2, acc);
      }
    }
    *yp = acc;
  }
}

template <typename T>
static int pbtrf_impl(char uplo, i64 n, i64 kd, T* AB, i64 ldab, i64* info, cudaStream_t s, const char* name) {
  const bool upper = (uplo == 'U' || uplo == 'u');
  if (!upper && !(uplo == 'L' || uplo == 'l')) return -1;
  if (n < 0) return -2;
  if (kd < 0) return -3;
  if (ldab < kd + 1) return -5;
  if (!info) return -6;
  if (n == 0) return cuda_status(cudaMemsetAsync(info, 0, sizeof(i64), s), name);
  const i64 bytes = (kd + 1) * (kd + 1) * (i64)sizeof(T);
  if (bytes > 227 * 1024 - 64) {
    set_error("%s: kd = %lld exceeds the shared-memory window (kd <= %d for this element size)", name, (long long)kd,
              sizeof(T) == 8 ? 167 : 237);
    return BM_ERR_UNSUPPORTED;
  }
  const void* fn = upper ? (const void*)pbtrf_kernel<T, true> : (const void*)pbtrf_kernel<T, false>;
  int r = cuda_status(ensure_smem(fn, (int)bytes), name);
  if (r) return r;
  if (upper)
    pbtrf_kernel<T, true><<<1, kPbThreads, (int)bytes, s>>>(n, (int)kd, AB, ldab, info);
  else
    pbtrf_kernel<T, false><<<1, kPbThreads, (int)bytes, s>>>(n, (int)kd, AB, ldab, info);
  return launch_status(name);
}

template <typename T>
static int pbtrs_impl(char uplo, i64 n, i64 kd, i64 nrhs, const T* AB, i64 ldab, T* B, i64 ldb, cudaStream_t s,
                      const char* name) {
  const bool upper = (uplo == 'U' || uplo == 'u');
  if (!upper && !(uplo == 'L' || uplo == 'l')) return -1;
  if (n < 0) return -2;
  if (kd < 0) return -3;
  if (nrhs < 0) return -4;
  if (ldab < kd + 1) return -6;
  if (ldb < std::max<i64>(1, n)) return -8;
  if (n == 0 || nrhs == 0) return BM_OK;
  int r = tbsv_general<T>(uplo, upper ? 'T' : 'N', 'N', n, kd, AB, ldab, B, 1, s, name, nrhs, ldb);
  if (r) return r;
  return tbsv_general<T>(uplo, upper ? 'N' : 'T', 'N', n, kd, AB, ldab, B, 1, s, name, nrhs, ldb);
}

template <typename T>
static int sbmv_impl(char uplo, i64 n, i64 k, T alpha, const T* A, i64 lda, const T* x, i64 incx, T beta, T* y,
                     i64 incy, cudaStream_t s, const char* name) {
  const bool upper = (uplo == 'U' || uplo == 'u');
  if (!upper && !(uplo == 'L' || uplo == 'l')) return -1;
  if (n < 0) return -2;
  if (k < 0) return -3;
  if (lda < k + 1) return -6;
  if (incx == 0) return -8;
  if (incy == 0) return -11;
  if (n == 0 || (alpha == T(0) && beta == T(1))) return BM_OK;
  if (k > 0x7fffffff) return -3;
  const int threads = 256;
  const i64 blocks = std::min<i64>(ceil_div(n, threads), (i64)num_sms() * 16);
  sbmv_kernel<T><<<(unsigned)blocks, threads, 0, s>>>(upper, n, (int)k, alpha, A, lda, x, incx, beta, y, incy);
  return launch_status(name);
}

}  // namespace bm

extern "C" int bm_dpbtrf(char uplo, int64_t n, int64_t kd, double* AB, int64_t ldab, int64_t* info,
                         bm_stream_t stream) {
  return bm::pbtrf_impl<double>(uplo, n, kd, AB, ldab, info, reinterpret_cast<cudaStream_t>(stream), "bm_dpbtrf");
}
extern "C" int bm_spbtrf(char uplo, int64_t n, int64_t kd, float* AB, int64_t ldab, int64_t* info, bm_stream_t stream) {
  return bm::pbtrf_impl<float>(uplo, n, kd, AB, ldab, info, reinterpret_cast<cudaStream_t>(stream), "bm_spbtrf");
}
extern "C" int bm_dpbtrs(char uplo, int64_t n, int64_t kd, int64_t nrhs, const double* AB, int64_t ldab, double* B,
                         int64_t ldb, bm_stream_t stream) {
  return bm::pbtrs_impl<double>(uplo, n, kd, nrhs, AB, ldab, B, ldb, reinterpret_cast<cudaStream_t>(stream),
                                "bm_dpbtrs");
}
extern "C" int bm_spbtrs(char uplo, int64_t n, int64_t kd, int64_t nrhs, const float* AB, int64_t ldab, float* B,
                         int64_t ldb, bm_stream_t stream) {
  return bm::pbtrs_impl<float>(uplo, n, kd, nrhs, AB, ldab, B, ldb, reinterpret_cast<cudaStream_t>(stream),
                               "bm_spbtrs");
}
extern "C" int bm_dsbmv(char uplo, int64_t n, int64_t k, double alpha, const double* A, int64_t lda, const double* x,
                        int64_t incx, double beta, double* y, int64_t incy, bm_stream_t stream) {
  return bm::sbmv_impl<double>(uplo, n, k, alpha, A, lda, x, incx, beta, y, incy,
                               reinterpret_cast<cudaStream_t>(stream), "bm_dsbmv");
}
extern "C" int bm_ssbmv(char uplo, int64_t n, int64_t k, float alpha, const float* A, int64_t lda, const float* x,
                        int64_t incx, float beta, float* y, int64_t incy, bm_stream_t stream) {
  return bm::sbmv_impl<float>(uplo, n, k, alpha, A, lda, x, incx, beta, y, incy,
                              reinterpret_cast<cudaStream_t>(stream), "bm_ssbmv");
}
