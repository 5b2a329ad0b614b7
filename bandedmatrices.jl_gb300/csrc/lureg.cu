// Register-window banded LU kernels (see lureg.cuh), one CTA per system.
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
  const unsigned threads = 32u * (unsigned)reg_warps(kl, ku);
  switch (cls) {
    case 4: gbtrf_reg_kernel<T, 4><<<1, threads, 0, stream>>>(m, n, (int)kl, (int)ku, ab, ldab, ipiv, info); break;
    case 8: gbtrf_reg_kernel<T, 8><<<1, threads, 0, stream>>>(m, n, (int)kl, (int)ku, ab, ldab, ipiv, info); break;
    case 16: gbtrf_reg_kernel<T, 16><<<1, threads, 0, stream>>>(m, n, (int)kl, (int)ku, ab, ldab, ipiv, info); break;
    case 32: gbtrf_reg_kernel<T, 32><<<1, threads, 0, stream>>>(m, n, (int)kl, (int)ku, ab, ldab, ipiv, info); break;
    case 64:
      if constexpr (reg_kl_max<T>() >= 64) {
        gbtrf_reg_kernel<T, 64><<<1, threads, 0, stream>>>(m, n, (int)kl, (int)ku, ab, ldab, ipiv, info);
        break;
      }
      [[fallthrough]];
    default:
      set_error("%s: band (%lld, %lld) outside the register-window classes", name, (long long)kl, (long long)ku);
      return BM_ERR_UNSUPPORTED;
  }
  return launch_status(name);
}

template int gbtrf_reg_run<float>(i64, i64, i64, i64, float*, i64, i64*, i64*, cudaStream_t, const char*);
template int gbtrf_reg_run<double>(i64, i64, i64, i64, double*, i64, i64*, i64*, cudaStream_t, const char*);

}  // namespace bm
