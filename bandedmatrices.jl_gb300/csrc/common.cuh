// Shared device/host helpers for the banded kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "../../include/bandedgpu.h"

namespace bm {

typedef int64_t i64;

// ---------------------------------------------------------------- host side
// Thread-local last-error text (bm_last_error()).
void set_error(const char* fmt, ...);

// Number of SMs of the current device (cached per device).
int num_sms();

// Opt a kernel into `bytes` of dynamic shared memory once per device.
cudaError_t ensure_smem(const void* kernel, int bytes);

// Address of this library's device status word on the current device.
int* status_word();

inline int cuda_status(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return BM_OK;
  set_error("%s: %s", where, cudaGetErrorString(e));
  return BM_ERR_CUDA;
}

// Checks the launch just enqueued and counts it (bm_launch_count).
int launch_status(const char* where);

inline i64 ceil_div(i64 a, i64 b) { return (a + b - 1) / b; }

// ---------------------------------------------------------------- device side
// Spin limits.  Every wait in these kernels is bounded, in polls and in time: on
// expiry the kernel records BM_STATUS_TIMEOUT in the status word and stops waiting.
constexpr uint32_t kSpinLimit = 1u << 26;

enum : int { BM_STATUS_TIMEOUT = 1 };

__device__ __forceinline__ void record_status(int* status, int code) {
  if (status) atomicOr(status, code);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Order this thread's generic-proxy shared-memory accesses before later
// async-proxy (bulk copy) writes to the same buffer.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// 1-D bulk copy global -> shared (TMA engine); src, dst 16-byte aligned and
// bytes a multiple of 16.  Completion is signalled on `bar` as tx bytes.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

// Nanoseconds of the GPU's global timer.
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// A poll of mbarrier.try_wait may suspend the thread for a hardware-chosen time, so a
// poll count alone does not bound a wait's duration: every wait also gives up after
// kWaitNs of global time.
constexpr uint64_t kWaitNs = 2000000000ull;

// Bounded wait for phase `phase` of `bar`: at most `limit` polls (never more than
// kSpinLimit) and at most kWaitNs.  Returns false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase, uint32_t limit = kSpinLimit) {
  if (limit > kSpinLimit) limit = kSpinLimit;
  if (mbar_try_wait(bar, phase)) return true;
  const uint64_t t0 = global_ns();
  for (uint32_t it = 1; it < limit; ++it) {
    if (mbar_try_wait(bar, phase)) return true;
    if ((it & 15) == 0 && global_ns() - t0 > kWaitNs) return false;
  }
  return false;
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may start before the previous kernel in the stream ends.
// grid_dep_wait() returns once every prerequisite grid has completed and its memory is
// visible; grid_dep_launch() lets the next such kernel start.  Both are no-ops for a
// kernel launched the ordinary way.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename T>
__device__ __forceinline__ T ldg(const T* p) {
  return __ldg(p);
}

// 1-D bulk copy shared -> global (TMA engine), tracked as a bulk group of the issuing
// thread; src, dst 16-byte aligned and bytes a multiple of 16.
__device__ __forceinline__ void bulk_s2g(void* dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the source shared memory of every committed bulk store may be reused
__device__ __forceinline__ void bulk_wait_read_all() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// every committed bulk store is complete
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// cp.async of one element (zero-filled when !valid), and its group commit / wait
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* src, bool valid) {
  const uint32_t d = smem_u32(dst);
  const int sz = valid ? (int)sizeof(T) : 0;
  if constexpr (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src), "r"(sz) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(sz) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

}  // namespace bm
