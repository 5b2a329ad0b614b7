// Adjoint of the banded solve X = A \ B (no counterpart in the reference; the
// ChainRules rrule of \ built beside ldiv!, src/banded/linalg.jl:24-47).
//
// For a loss L with upstream gradient W = dL/dX:
//     dL/dB = A^{-T} W                  (xGBTRS 'T' on the stored factors -- the
//                                        transposed solve of linalg.jl:41-47)
//     dL/dA = -(A^{-T} W) X^T  on the band of A only (entries outside the band are
//                                        structurally zero and get no gradient)
// X is either passed in or, when memory is tight, recomputed from B with one more
// xGBTRS 'N' into caller-provided workspace.  The band gradient is written in BLAS
// band layout ((kl+ku+1) x n, leading dim ldg), one thread per band entry, summing
// the right-hand sides in ascending order: an HBM-bound stream.
#include "lu.cuh"

namespace bm {

template <typename T>
__global__ void band_outer_kernel(i64 n, int kl, int ku, i64 nrhs, const T* __restrict__ lam, i64 ldl,
                                  const T* __restrict__ x, i64 ldx, T* __restrict__ g, i64 ldg) {
  const int rows = kl + ku + 1;
  const i64 total = n * (i64)rows;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
    const i64 j = e / rows;
    const int r = (int)(e - j * rows);
    const i64 i = j + r - ku;
    T acc = T(0);
    if (i >= 0 && i < n)
      for (i64 c = 0; c < nrhs; ++c) acc = fma(-lam[i + c * ldl], x[j + c * ldx], acc);
    g[r + j * ldg] = acc;
  }
}

template <typename T>
static int gb_adjoint_impl(i64 n, i64 kl, i64 ku, i64 nrhs, const T* lu, i64 ldab, const i64* ipiv, const T* X,
                           const T* B, const T* W, T* gB, T* gband, i64 ldg, T* Xwork, cudaStream_t stream,
                           const char* name);

}  // namespace bm

// forward declarations of the library's own solve entry points
extern "C" int bm_dgbtrs(char, int64_t, int64_t, int64_t, int64_t, const double*, int64_t, const int64_t*, double*,
                         int64_t, bm_stream_t);
extern "C" int bm_sgbtrs(char, int64_t, int64_t, int64_t, int64_t, const float*, int64_t, const int64_t*, float*,
                         int64_t, bm_stream_t);

namespace bm {

template <typename T>
static int trs(char t, i64 n, i64 kl, i64 ku, i64 nrhs, const T* ab, i64 ldab, const i64* ipiv, T* b, i64 ldb,
               cudaStream_t s) {
  if constexpr (sizeof(T) == 8)
    return bm_dgbtrs(t, n, kl, ku, nrhs, ab, ldab, ipiv, b, ldb, reinterpret_cast<bm_stream_t>(s));
  else
    return bm_sgbtrs(t, n, kl, ku, nrhs, ab, ldab, ipiv, b, ldb, reinterpret_cast<bm_stream_t>(s));
}

template <typename T>
static int gb_adjoint_impl(i64 n, i64 kl, i64 ku, i64 nrhs, const T* lu, i64 ldab, const i64* ipiv, const T* X,
                           const T* B, const T* W, T* gB, T* gband, i64 ldg, T* Xwork, cudaStream_t stream,
                           const char* name) {
  if (n < 0) return -1;
  if (kl < 0) return -2;
  if (ku < 0) return -3;
  if (nrhs < 0) return -4;
  const bool work = n > 0 && nrhs > 0;  // the pointers are read only when there is work
  if (!lu && work) return -5;
  if (ldab < 2 * kl + ku + 1) return -6;
  if (!ipiv && work) return -7;
  if (!X && (!B || !Xwork) && work) return -8;
  if (!W && work) return -10;
  if (!gB && work) return -11;
  if (ldg < kl + ku + 1) return -13;
  if (n == 0 || nrhs == 0) return BM_OK;
  const size_t bytes = sizeof(T) * (size_t)n * (size_t)nrhs;
  // dL/dB = A^{-T} W
  int r = cuda_status(cudaMemcpyAsync(gB, W, bytes, cudaMemcpyDeviceToDevice, stream), name);
  if (r) return r;
  r = trs<T>('T', n, kl, ku, nrhs, lu, ldab, ipiv, gB, n, stream);
  if (r) return r;
  // X, recomputed when not kept
  if (!X) {
    r = cuda_status(cudaMemcpyAsync(Xwork, B, bytes, cudaMemcpyDeviceToDevice, stream), name);
    if (r) return r;
    r = trs<T>('N', n, kl, ku, nrhs, lu, ldab, ipiv, Xwork, n, stream);
    if (r) return r;
    X = Xwork;
  }
  if (gband) {
    const i64 total = n * (kl + ku + 1);
    const i64 blocks = std::min<i64>(ceil_div(total, 256), (i64)num_sms() * 16);
    band_outer_kernel<T><<<(unsigned)blocks, 256, 0, stream>>>(n, (int)kl, (int)ku, nrhs, gB, n, X, n, gband, ldg);
    r = launch_status(name);
  }
  return r;
}

}  // namespace bm

extern "C" int bm_dgbsv_adjoint(int64_t n, int64_t kl, int64_t ku, int64_t nrhs, const double* LU, int64_t ldab,
                                const int64_t* ipiv, const double* X, const double* B, const double* W,
                                double* grad_B, double* grad_band, int64_t ldg, double* Xwork, bm_stream_t stream) {
  return bm::gb_adjoint_impl<double>(n, kl, ku, nrhs, LU, ldab, ipiv, X, B, W, grad_B, grad_band, ldg, Xwork,
                                     reinterpret_cast<cudaStream_t>(stream), "bm_dgbsv_adjoint");
}
extern "C" int bm_sgbsv_adjoint(int64_t n, int64_t kl, int64_t ku, int64_t nrhs, const float* LU, int64_t ldab,
                                const int64_t* ipiv, const float* X, const float* B, const float* W, float* grad_B,
                                float* grad_band, int64_t ldg, float* Xwork, bm_stream_t stream) {
  return bm::gb_adjoint_impl<float>(n, kl, ku, nrhs, LU, ldab, ipiv, X, B, W, grad_B, grad_band, ldg, Xwork,
                                    reinterpret_cast<cudaStream_t>(stream), "bm_sgbsv_adjoint");
}
