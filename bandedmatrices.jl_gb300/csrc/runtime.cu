// Host runtime of the library: error text, device properties, status word.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <mutex>
#include <utility>

#include "common.cuh"

namespace bm {

static thread_local char g_err[512] = {0};

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

static std::mutex g_mu;
static std::atomic<unsigned long long> g_launches{0};

int launch_status(const char* where) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return cuda_status(cudaGetLastError(), where);
}

int num_sms() {
  static std::map<int, int> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = cache.find(dev);
  if (it != cache.end()) return it->second;
  int v = 0;
  cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
  if (v <= 0) v = 1;
  cache[dev] = v;
  return v;
}

cudaError_t ensure_smem(const void* kernel, int bytes) {
  static std::map<std::pair<const void*, int>, int> done;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_mu);
  auto key = std::make_pair(kernel, dev);
  auto it = done.find(key);
  if (it != done.end() && it->second >= bytes) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) done[key] = bytes;
  return e;
}

// One status word per device, in this module's static device memory.
static __device__ int g_status_word;

int* status_word() {
  static std::map<int, int*> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = cache.find(dev);
  if (it != cache.end()) return it->second;
  int* p = nullptr;
  if (cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_status_word) != cudaSuccess) p = nullptr;
  cache[dev] = p;
  return p;
}

}  // namespace bm

extern "C" int bm_version(void) { return 100; }

extern "C" const char* bm_last_error(void) { return bm::g_err; }

extern "C" int bm_device_status(int* status_out, int clear, bm_stream_t stream) {
  if (!status_out) return -1;
  int* w = bm::status_word();
  if (!w) {
    bm::set_error("bm_device_status: status word unavailable");
    return BM_ERR_CUDA;
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int r = bm::cuda_status(cudaMemcpyAsync(status_out, w, sizeof(int), cudaMemcpyDeviceToHost, s),
                          "bm_device_status");
  if (r) return r;
  if (clear) {
    r = bm::cuda_status(cudaMemsetAsync(w, 0, sizeof(int), s), "bm_device_status");
    if (r) return r;
  }
  return bm::cuda_status(cudaStreamSynchronize(s), "bm_device_status");
}

// Bounded-wait self-test: one thread waits, through the same mbar_wait the streaming
// kernels use, for a phase of an mbarrier that nothing arrives at.  The wait gives up
// after `limit` polls, the kernel records BM_STATUS_TIMEOUT in the status word and
// returns, and the context stays usable.  `done` (device int) is set to 1 when the
// kernel has returned from its wait.
namespace bm {
__global__ void wait_selftest_kernel(uint32_t limit, int* status, int* done) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    if (!mbar_wait(&bar, 0u, limit)) record_status(status, BM_STATUS_TIMEOUT);
    *done = 1;
  }
}
}  // namespace bm

extern "C" int bm_wait_selftest(int64_t spin_limit, int* done, bm_stream_t stream) {
  if (spin_limit < 1 || spin_limit > (int64_t)bm::kSpinLimit) return -1;
  if (!done) return -2;
  int* w = bm::status_word();
  if (!w) {
    bm::set_error("bm_wait_selftest: status word unavailable");
    return BM_ERR_CUDA;
  }
  bm::wait_selftest_kernel<<<1, 32, 0, reinterpret_cast<cudaStream_t>(stream)>>>((uint32_t)spin_limit, w, done);
  return bm::launch_status("bm_wait_selftest");
}

// Kernels this library has enqueued in the process (captured launches included).
extern "C" unsigned long long bm_launch_count(void) { return bm::g_launches.load(std::memory_order_relaxed); }
