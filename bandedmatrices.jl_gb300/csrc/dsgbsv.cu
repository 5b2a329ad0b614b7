// Single-system mixed-precision refined banded solve (bm_dsgbsv): LAPACK DSGESV's
// scheme on band storage, with the whole refinement loop on the device.
//
// No counterpart in the reference; it replaces lu! + ldiv! (src/banded/BandedLU.jl:
// 90-103, src/banded/linalg.jl:24-30) for a caller that accepts a backward-error
// target.  For a band with 64 <= kl + ku <= 256 (kl <= 224) the FP32 factorization is
// the tensor-core blocked LU of tclu.cuh; narrower bands take the FP32 dgbtf2-order
// factorization of lu.cu.  Then, with the FP32 factors:
//     x = FP64(LU32 \ FP32(b))
//     k = 0, 1, ...: r = b - A x (FP64, the original band, bm_dgbmv's kernels)
//                    berr = max_c ||r_c||_inf / (||A||_inf ||x_c||_inf + ||b_c||_inf)
//                    stop when berr <= tol or k == maxit
//                    x += FP64(LU32 \ FP32(r))
// The host enqueues every launch up front; a device flag set by the check kernel
// turns the remaining launches into no-ops, so the call never synchronises.
#include "bandsolve.cuh"
#include "mixedlu.cuh"
#include "tclu.cuh"

namespace bm {

int dgbmv_flagged(char trans, i64 m, i64 n, i64 kl, i64 ku, double alpha, const double* A, i64 lda, const double* x,
                  i64 incx, double beta, double* y, i64 incy, const int* skip, cudaStream_t stream, const char* name);

namespace {

// Control words after the FP64 residual in `work` (unsigned long long):
//   [0] ||A||_inf (bits), [1] done flag (int, low word), [2, 2+nrhs) ||b_c||_inf,
//   [2+nrhs, 2+2nrhs) ||r_c||_inf, [2+2nrhs, 2+3nrhs) ||x_c||_inf (bits; every value
//   is >= 0, so the bit patterns order as the numbers, NaN above all)
__device__ __forceinline__ unsigned long long abits(double v) { return (unsigned long long)__double_as_longlong(fabs(v)); }
__device__ __forceinline__ unsigned long long bmax(unsigned long long a, unsigned long long b) { return a > b ? a : b; }

template <int NT>
__device__ __forceinline__ unsigned long long block_max(unsigned long long v, unsigned long long* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 16; o; o >>= 1) v = bmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = 1; k < NT / 32; ++k) v = bmax(v, red[k]);
  return v;
}

constexpr int kDsThreads = 256;

// ||A||_inf (row sums of |A|, FP64) and ||b_c||_inf; W zeroed before.
__global__ void __launch_bounds__(kDsThreads) ds_norms_kernel(i64 n, int kl, int ku, i64 nrhs, const double* A,
                                                              i64 lda, const double* B, i64 ldb,
                                                              unsigned long long* W) {
  __shared__ unsigned long long red[kDsThreads / 32];
  unsigned long long m = 0;
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const i64 c0 = max((i64)0, i - kl), c1 = min(n - 1, i + ku);
    double s = 0.0;
    for (i64 c = c0; c <= c1; ++c) s += fabs(A[(ku + i - c) + c * lda]);
    m = bmax(m, abits(s));
  }
  m = block_max<kDsThreads>(m, red);
  if (threadIdx.x == 0) atomicMax(W, m);
  for (i64 c = 0; c < nrhs; ++c) {
    unsigned long long b = 0;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
      b = bmax(b, abits(B[i + c * ldb]));
    b = block_max<kDsThreads>(b, red);
    if (threadIdx.x == 0) atomicMax(W + 2 + c, b);
  }
}

// FP64 band (kl+ku+1 rows) -> FP32 gbtrf storage (2kl+ku+1 rows, fill rows zero).
__global__ void ds_round_kernel(i64 n, int kl, int ku, const double* A, i64 lda, float* F, i64 ldf) {
  const i64 rows = 2 * (i64)kl + ku + 1, tot = rows * n;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
    const i64 c = e / rows, r = e - c * rows;
    F[r + c * ldf] = r < kl ? 0.0f : (float)A[(r - kl) + c * lda];
  }
}

// A failed FP32 factorization: no solve, no refinement.
__global__ void ds_after_factor_kernel(const i64* info, unsigned long long* W, int32_t* iter, double* berr) {
  if (*info != 0) {
    *reinterpret_cast<int*>(W + 1) = 1;
    *iter = 0;
    *berr = __longlong_as_double(0x7ff0000000000000LL);  // +inf: not solved
  }
}

// R32 = FP32(B) (leading dim n) before the first solve.
__global__ void ds_b_to_r32_kernel(i64 n, i64 nrhs, const double* B, i64 ldb, float* R32,
                                   const unsigned long long* W) {
  if (*reinterpret_cast<volatile const int*>(W + 1)) return;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < n * nrhs; e += (i64)gridDim.x * blockDim.x) {
    const i64 c = e / n, i = e - c * n;
    R32[e] = (float)B[i + c * ldb];
  }
}

// X = FP64(R32) (first solve) or X += FP64(R32) (correction).
__global__ void ds_update_kernel(i64 n, i64 nrhs, const float* R32, double* X, i64 ldx, int first,
                                 const unsigned long long* W) {
  if (*reinterpret_cast<volatile const int*>(W + 1)) return;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < n * nrhs; e += (i64)gridDim.x * blockDim.x) {
    const i64 c = e / n, i = e - c * n;
    const double d = (double)R32[e];
    X[i + c * ldx] = first ? d : X[i + c * ldx] + d;
  }
}

// R = B (leading dim n), and the residual / solution maxima reset.
__global__ void ds_copy_b_kernel(i64 n, i64 nrhs, const double* B, i64 ldb, double* R, unsigned long long* W) {
  if (*reinterpret_cast<volatile const int*>(W + 1)) return;
  if (blockIdx.x == 0)
    for (i64 c = threadIdx.x; c < 2 * nrhs; c += blockDim.x) W[2 + nrhs + c] = 0ull;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < n * nrhs; e += (i64)gridDim.x * blockDim.x) {
    const i64 c = e / n, i = e - c * n;
    R[e] = B[i + c * ldb];
  }
}

// ||r_c||_inf and ||x_c||_inf.
__global__ void __launch_bounds__(kDsThreads) ds_reduce_kernel(i64 n, i64 nrhs, const double* R, const double* X,
                                                               i64 ldx, unsigned long long* W) {
  if (*reinterpret_cast<volatile const int*>(W + 1)) return;
  __shared__ unsigned long long red[kDsThreads / 32];
  for (i64 c = 0; c < nrhs; ++c) {
    unsigned long long r = 0, x = 0;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
      r = bmax(r, abits(R[i + c * n]));
      x = bmax(x, abits(X[i + c * ldx]));
    }
    r = block_max<kDsThreads>(r, red);
    if (threadIdx.x == 0) atomicMax(W + 2 + nrhs + c, r);
    x = block_max<kDsThreads>(x, red);
    if (threadIdx.x == 0) atomicMax(W + 2 + 2 * nrhs + c, x);
  }
}

// The backward error after k corrections; stop (set the flag) when it meets tol or k
// reached maxit (a NaN stops too); otherwise R32 = FP32(r) for the next correction.
__global__ void ds_check_kernel(i64 n, i64 nrhs, int k, int maxit, double tol, const double* R, float* R32,
                                unsigned long long* W, int32_t* iter, double* berr) {
  if (*reinterpret_cast<volatile const int*>(W + 1)) return;
  const double anorm = __longlong_as_double((long long)W[0]);
  double be = 0.0;
  for (i64 c = 0; c < nrhs; ++c) {
    const double rm = __longlong_as_double((long long)W[2 + nrhs + c]);
    const double xm = __longlong_as_double((long long)W[2 + 2 * nrhs + c]);
    const double bm = __longlong_as_double((long long)W[2 + c]);
    const double den = anorm * xm + bm;
    const double bc = den > 0.0 ? rm / den : rm;
    be = (bc > be || bc != bc) ? bc : be;
  }
  const bool stop = !(be > tol) || k >= maxit;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *berr = be;
    *iter = k;
    if (stop) *reinterpret_cast<int*>(W + 1) = 1;
  }
  if (stop) return;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < n * nrhs; e += (i64)gridDim.x * blockDim.x)
    R32[e] = (float)R[e];
}

// gbtrs 'N' with the FP32 factors (ldf a multiple of 4): one CTA of kBsWarps warps per
// right-hand side of R32 (leading dim n), the sweeps of bandsolve.cuh.  A sweep whose
// wait ran out ends the CTA (its copies landed): the status word reports it.
__global__ void __launch_bounds__(32 * kBsWarps) ds_solve_kernel(i64 n, int kl, int ku, i64 nrhs, const float* F,
                                                                 i64 ldf, const i64* ipiv, float* R32,
                                                                 const unsigned long long* W, int* status) {
  if (*reinterpret_cast<volatile const int*>(W + 1)) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);  // forward slots, then backward slots
  const int stages = bs_stages(ldf);
  for (i64 c = blockIdx.x; c < nrhs; c += gridDim.x) {
    if (threadIdx.x == 0) {
      for (int q = 0; q < 8; ++q) mbar_init(&bars[q], 1);
      fence_mbar_init();
    }
    __syncthreads();
    float* b = R32 + c * n;
    const bool ok = bs_sweep<true>(n, kl, ku, F, ldf, ipiv, b, smem_raw, bars, stages, status) &&
                    bs_sweep<false>(n, kl, ku, F, ldf, ipiv, b, smem_raw, bars + 4, stages, status);
    __syncthreads();
    if (threadIdx.x == 0)
      for (int q = 0; q < 8; ++q)
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&bars[q])) : "memory");
    __syncthreads();
    if (!ok) return;
  }
}

int sgbtrf_tc_run(i64 n, i64 kl, i64 ku, const double* A, i64 lda, float* F, i64 ldf, i64* ipiv, i64* info,
                  cudaStream_t stream, const char* name) {
  const int bytes = tc_smem_bytes((int)kl);
  int r = cuda_status(ensure_smem((const void*)sgbtrf_tc_kernel, bytes), name);
  if (r) return r;
  sgbtrf_tc_kernel<<<1, kTcThreads, bytes, stream>>>(n, (int)kl, (int)ku, A, lda, F, ldf, ipiv, info, status_word());
  return launch_status(name);
}

}  // namespace

static int dsgbsv_impl(i64 n, i64 kl, i64 ku, i64 nrhs, const double* AB, i64 ldab, const double* B, i64 ldb,
                       double* X, i64 ldx, i64* ipiv, float* swork, double* work, double tol, i64 maxit,
                       int32_t* iter, double* berr, i64* info, cudaStream_t s, const char* name) {
  if (n < 0) return -1;
  if (kl < 0) return -2;
  if (ku < 0) return -3;
  if (nrhs < 0) return -4;
  if (!AB && n > 0) return -5;
  if (ldab < kl + ku + 1) return -6;
  if (!B && n * nrhs > 0) return -7;
  if (ldb < std::max<i64>(1, n)) return -8;
  if (!X && n * nrhs > 0) return -9;
  if (ldx < std::max<i64>(1, n)) return -10;
  if (!ipiv && n > 0) return -11;
  if (!swork && n > 0) return -12;
  if (reinterpret_cast<uintptr_t>(swork) & 15) return BM_ERR_ALIGN;
  if (!work && n * nrhs > 0) return -13;
  if (!(tol >= 0.0)) return -14;
  if (maxit < 0) return -15;
  if (!iter) return -16;
  if (!berr) return -17;
  if (!info) return -18;
  if (kl + ku > 256) {
    set_error("%s: kl + ku = %lld exceeds the refined solve's limit of 256", name, (long long)(kl + ku));
    return BM_ERR_UNSUPPORTED;
  }
  int r;
  const int mx = (int)std::min<i64>(maxit, 100);
  if ((r = cuda_status(cudaMemsetAsync(info, 0, sizeof(i64), s), name))) return r;
  if ((r = cuda_status(cudaMemsetAsync(iter, 0, sizeof(int32_t), s), name))) return r;
  if ((r = cuda_status(cudaMemsetAsync(berr, 0, sizeof(double), s), name))) return r;
  if (n == 0 || nrhs == 0) {
    if (n > 0) {  // factor only
      const i64 ldf = (2 * kl + ku + 1 + 3) & ~(i64)3;
      if (tc_lu_fits(kl, ku)) return sgbtrf_tc_run(n, kl, ku, AB, ldab, swork, ldf, ipiv, info, s, name);
      const int blocks = (int)std::min<i64>(ceil_div(ldf * n, 256), (i64)num_sms() * 8);
      ds_round_kernel<<<blocks, 256, 0, s>>>(n, (int)kl, (int)ku, AB, ldab, swork, ldf);
      if ((r = launch_status(name))) return r;
      return bm_sgbtrf(n, n, kl, ku, swork, ldf, ipiv, info, reinterpret_cast<bm_stream_t>(s));
    }
    return BM_OK;
  }
  const i64 ldf = (2 * kl + ku + 1 + 3) & ~(i64)3;  // a multiple of 4: 16-byte column segments
  float* F = swork;
  float* R32 = swork + ldf * n;
  double* R = work;
  unsigned long long* W = reinterpret_cast<unsigned long long*>(work + n * nrhs);
  const int* done = reinterpret_cast<const int*>(W + 1);
  const int nsm = num_sms();
  const int eblocks = (int)std::min<i64>(ceil_div(n * nrhs, 256), (i64)nsm * 8);
  const int rblocks = (int)std::min<i64>(ceil_div(n, kDsThreads), (i64)nsm * 4);

  if ((r = cuda_status(cudaMemsetAsync(W, 0, (2 + 3 * nrhs) * sizeof(unsigned long long), s), name))) return r;
  ds_norms_kernel<<<rblocks, kDsThreads, 0, s>>>(n, (int)kl, (int)ku, nrhs, AB, ldab, B, ldb, W);
  if ((r = launch_status(name))) return r;
  // ---- FP32 factorization
  if (tc_lu_fits(kl, ku)) {
    if ((r = sgbtrf_tc_run(n, kl, ku, AB, ldab, F, ldf, ipiv, info, s, name))) return r;
  } else {
    const int blocks = (int)std::min<i64>(ceil_div(ldf * n, 256), (i64)nsm * 8);
    ds_round_kernel<<<blocks, 256, 0, s>>>(n, (int)kl, (int)ku, AB, ldab, F, ldf);
    if ((r = launch_status(name))) return r;
    if ((r = bm_sgbtrf(n, n, kl, ku, F, ldf, ipiv, info, reinterpret_cast<bm_stream_t>(s)))) return r;
  }
  ds_after_factor_kernel<<<1, 1, 0, s>>>(info, W, iter, berr);
  if ((r = launch_status(name))) return r;
  // ---- first solve
  const int ssmem = bs_smem_bytes(ldf);
  if ((r = cuda_status(ensure_smem((const void*)ds_solve_kernel, ssmem), name))) return r;
  const int sblocks = (int)std::min<i64>(nrhs, (i64)nsm);
  ds_b_to_r32_kernel<<<eblocks, 256, 0, s>>>(n, nrhs, B, ldb, R32, W);
  if ((r = launch_status(name))) return r;
  ds_solve_kernel<<<sblocks, 32 * kBsWarps, ssmem, s>>>(n, (int)kl, (int)ku, nrhs, F, ldf, ipiv, R32, W, status_word());
  if ((r = launch_status(name))) return r;
  ds_update_kernel<<<eblocks, 256, 0, s>>>(n, nrhs, R32, X, ldx, 1, W);
  if ((r = launch_status(name))) return r;
  // ---- refinement: every launch enqueued now, no-ops once the flag is set
  for (int k = 0; k <= mx; ++k) {
    ds_copy_b_kernel<<<eblocks, 256, 0, s>>>(n, nrhs, B, ldb, R, W);
    if ((r = launch_status(name))) return r;
    for (i64 c = 0; c < nrhs; ++c)
      if ((r = dgbmv_flagged('N', n, n, kl, ku, -1.0, AB, ldab, X + c * ldx, 1, 1.0, R + c * n, 1, done, s, name)))
        return r;
    ds_reduce_kernel<<<rblocks, kDsThreads, 0, s>>>(n, nrhs, R, X, ldx, W);
    if ((r = launch_status(name))) return r;
    ds_check_kernel<<<eblocks, 256, 0, s>>>(n, nrhs, k, mx, tol, R, R32, W, iter, berr);
    if ((r = launch_status(name))) return r;
    if (k == mx) break;
    ds_solve_kernel<<<sblocks, 32 * kBsWarps, ssmem, s>>>(n, (int)kl, (int)ku, nrhs, F, ldf, ipiv, R32, W, status_word());
    if ((r = launch_status(name))) return r;
    ds_update_kernel<<<eblocks, 256, 0, s>>>(n, nrhs, R32, X, ldx, 0, W);
    if ((r = launch_status(name))) return r;
  }
  return BM_OK;
}

// FP32 factorization alone (the first step of bm_dsgbsv), for tests and profiling.
static int sgbtrf_mixed_impl(i64 n, i64 kl, i64 ku, const double* AB, i64 ldab, float* F, i64 ldf, i64* ipiv,
                             i64* info, cudaStream_t s, const char* name) {
  if (n < 0) return -1;
  if (kl < 0) return -2;
  if (ku < 0) return -3;
  if (!AB && n > 0) return -4;
  if (ldab < kl + ku + 1) return -5;
  if (!F && n > 0) return -6;
  if (ldf < 2 * kl + ku + 1) return -7;
  if (!ipiv && n > 0) return -8;
  if (!info) return -9;
  if (!tc_lu_fits(kl, ku)) {
    set_error("%s: the tensor-core factorization needs 64 <= kl + ku <= 256 and kl <= 224", name);
    return BM_ERR_UNSUPPORTED;
  }
  if (n == 0) return cuda_status(cudaMemsetAsync(info, 0, sizeof(i64), s), name);
  return sgbtrf_tc_run(n, kl, ku, AB, ldab, F, ldf, ipiv, info, s, name);
}

}  // namespace bm

extern "C" int bm_dsgbsv(int64_t n, int64_t kl, int64_t ku, int64_t nrhs, const double* AB, int64_t ldab,
                         const double* B, int64_t ldb, double* X, int64_t ldx, int64_t* ipiv, float* swork,
                         double* work, double tol, int64_t maxit, int32_t* iter, double* berr, int64_t* info,
                         bm_stream_t stream) {
  return bm::dsgbsv_impl(n, kl, ku, nrhs, AB, ldab, B, ldb, X, ldx, ipiv, swork, work, tol, maxit, iter, berr, info,
                         reinterpret_cast<cudaStream_t>(stream), "bm_dsgbsv");
}

extern "C" int bm_sgbtrf_tc(int64_t n, int64_t kl, int64_t ku, const double* AB, int64_t ldab, float* F, int64_t ldf,
                            int64_t* ipiv, int64_t* info, bm_stream_t stream) {
  return bm::sgbtrf_mixed_impl(n, kl, ku, AB, ldab, F, ldf, ipiv, info, reinterpret_cast<cudaStream_t>(stream),
                               "bm_sgbtrf_tc");
}
