// Arithmetic-pipe probe: the fma rate this GPU sustains in Float64 or Float32.  It is
// the compute roof of the kernels the FP64 pipe bounds (gbmv and gbmm in Float64, the
// FP64 residuals, the plain batched solve): on a GB300 the FP64 rate is a small
// fraction of the Float32 rate, so these kernels sit below the HBM roofline.
// Each thread runs 8 independent fma chains (enough to cover the pipe latency) and
// writes nothing unless the chains reach an impossible value.
#include "common.cuh"

namespace bm {

template <typename T>
__global__ void __launch_bounds__(256) fma_probe_kernel(int iters, T a, T b, T* sink) {
  T v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = (T)(threadIdx.x + i) * T(1e-3);
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = fma(v[i], a, b);
  T s = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += v[i];
  if (s == T(-1234.5)) *sink = s;
}

static __device__ double g_sink64;
static __device__ float g_sink32;

template <typename T>
static int probe(double* fma_per_s, cudaStream_t stream) {
  T* d_sink = nullptr;
  int r;
  if constexpr (sizeof(T) == 8) r = cuda_status(cudaGetSymbolAddress((void**)&d_sink, g_sink64), "bm_probe_fma_rate");
  else r = cuda_status(cudaGetSymbolAddress((void**)&d_sink, g_sink32), "bm_probe_fma_rate");
  if (r) return r;
  const int blocks = num_sms() * 8, threads = 256, iters = sizeof(T) == 8 ? (1 << 11) : (1 << 15);
  cudaEvent_t e0, e1;
  if ((r = cuda_status(cudaEventCreate(&e0), "bm_probe_fma_rate"))) return r;
  if ((r = cuda_status(cudaEventCreate(&e1), "bm_probe_fma_rate"))) {
    cudaEventDestroy(e0);
    return r;
  }
  fma_probe_kernel<T><<<blocks, threads, 0, stream>>>(64, T(0.999), T(1e-4), d_sink);  // warm-up
  r = launch_status("bm_probe_fma_rate");
  float best = 0.f;
  for (int rep = 0; rep < 3 && !r; ++rep) {
    cudaEventRecord(e0, stream);
    fma_probe_kernel<T><<<blocks, threads, 0, stream>>>(iters, T(0.999), T(1e-4), d_sink);
    r = launch_status("bm_probe_fma_rate");
    cudaEventRecord(e1, stream);
    if (!r) r = cuda_status(cudaEventSynchronize(e1), "bm_probe_fma_rate");
    float ms = 0.f;
    if (!r) cudaEventElapsedTime(&ms, e0, e1);
    if (ms > 0.f && (best == 0.f || ms < best)) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (r) return r;
  *fma_per_s = best > 0.f ? (double)blocks * threads * 8.0 * iters / (best * 1e-3) : 0.0;
  return BM_OK;
}

}  // namespace bm

extern "C" int bm_probe_fma_rate(int elem_bytes, double* fma_per_s, bm_stream_t stream) {
  if (!fma_per_s) return -2;
  if (elem_bytes == 8) return bm::probe<double>(fma_per_s, reinterpret_cast<cudaStream_t>(stream));
  if (elem_bytes == 4) return bm::probe<float>(fma_per_s, reinterpret_cast<cudaStream_t>(stream));
  return -1;
}
