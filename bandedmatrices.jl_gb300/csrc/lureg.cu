// Register-window banded LU kernels (see lureg.cuh), one CTA per system.
#include <algorithm>

#include "lureg.cuh"

namespace bm {

// Two CTAs' worth of registers per SM for the larger classes (at most 128 per thread):
// the scheduler otherwise hoists every multiplier load of a step ahead of the update.
template <typename T, int KL>
__global__ void __launch_bounds__(32 * kRegMaxWarps, KL >= 32 ? 2 : 1)
    gbtrf_reg_kernel(i64 m, i64 n, int kl, int ku, T* ab, i64 ldab, i64* ipiv, i64* info) {
  __shared__ RegShared<T, KL, 32 * kRegMaxWarps> sh;
  const i64 r = gbtrf_reg<T, KL, 32 * kRegMaxWarps>(m, n, kl, ku, ab, ldab, ipiv, sh, (int)threadIdx.x, (int)blockDim.x, blockDim.x > 32);
  if (threadIdx.x == 0) *info = r;
}

template <typename T>
int gbtrf_reg_run(i64 m, i64 n, i64 kl, i64 ku, T* ab, i64 ldab, i64* ipiv, i64* info, cudaStream_t stream,
                  const char* name) {
  const int cls = reg_class<T>(kl, ku);
  if (!cls) {
    set_error("%s: band (%lld, %lld) outside the register-window classes", name, (long long)kl, (long long)ku);
    return BM_ERR_UNSUPPORTED;
  }
  const unsigned threads = 32u * (unsigned)reg_warps(kl, ku);
  reg_dispatch<reg_kl_max<T>()>(cls, [&](auto k) {
    gbtrf_reg_kernel<T, decltype(k)::v><<<1, threads, 0, stream>>>(m, n, (int)kl, (int)ku, ab, ldab, ipiv, info);
    return 0;
  });
  return launch_status(name);
}

template <typename T, int KL>
__global__ void __launch_bounds__(32) gbtrs_reg_fwd_kernel(i64 n, int kl, int ku, i64 nrhs, const T* ab, i64 ldab,
                                                           const i64* ipiv, T* B, i64 ldb) {
  __shared__ RegFwdStage<T, KL> st[2];
  for (i64 r0 = (i64)blockIdx.x * 32; r0 < nrhs; r0 += (i64)gridDim.x * 32)
    gbtrs_reg_fwd<T, KL>(n, kl, ku, (int)min((i64)32, nrhs - r0), ab, ldab, ipiv, B + r0 * ldb, ldb, st,
                         (int)threadIdx.x);
}

template <typename T, int KV>
__global__ void __launch_bounds__(32) gbtrs_reg_bwd_kernel(i64 n, int kv, i64 nrhs, const T* ab, i64 ldab, T* B,
                                                           i64 ldb) {
  __shared__ RegBwdStage<T, KV> st[2];
  for (i64 r0 = (i64)blockIdx.x * 32; r0 < nrhs; r0 += (i64)gridDim.x * 32)
    gbtrs_reg_bwd<T, KV>(n, kv, (int)min((i64)32, nrhs - r0), ab, ldab, B + r0 * ldb, ldb, st, (int)threadIdx.x);
}

template <typename T>
int gbtrs_reg_run(i64 n, i64 kl, i64 ku, i64 nrhs, const T* ab, i64 ldab, const i64* ipiv, T* B, i64 ldb,
                  cudaStream_t stream, const char* name) {
  if (!reg_solve_fits<T>(kl, ku)) {
    set_error("%s: band (%lld, %lld) outside the register-window classes", name, (long long)kl, (long long)ku);
    return BM_ERR_UNSUPPORTED;
  }
  const unsigned grid = (unsigned)std::min<i64>(ceil_div(nrhs, (i64)32), 65535);
  if (kl > 0) {
    reg_dispatch<reg_kl_max<T>()>(reg_class<T>(kl, 0), [&](auto k) {
      gbtrs_reg_fwd_kernel<T, decltype(k)::v><<<grid, 32, 0, stream>>>(n, (int)kl, (int)ku, nrhs, ab, ldab, ipiv, B, ldb);
      return 0;
    });
    if (int r = launch_status(name)) return r;
  }
  reg_dispatch<2 * reg_kl_max<T>()>(reg_kv_class<T>(kl + ku), [&](auto k) {
    gbtrs_reg_bwd_kernel<T, decltype(k)::v><<<grid, 32, 0, stream>>>(n, (int)(kl + ku), nrhs, ab, ldab, B, ldb);
    return 0;
  });
  return launch_status(name);
}

template int gbtrs_reg_run<float>(i64, i64, i64, i64, const float*, i64, const i64*, float*, i64, cudaStream_t,
                                  const char*);
template int gbtrs_reg_run<double>(i64, i64, i64, i64, const double*, i64, const i64*, double*, i64, cudaStream_t,
                                   const char*);
template int gbtrf_reg_run<float>(i64, i64, i64, i64, float*, i64, i64*, i64*, cudaStream_t, const char*);
template int gbtrf_reg_run<double>(i64, i64, i64, i64, double*, i64, i64*, i64*, cudaStream_t, const char*);

}  // namespace bm
