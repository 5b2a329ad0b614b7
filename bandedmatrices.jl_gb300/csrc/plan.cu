// Plans for the batched solves: the autotuned launch schedule and its workspace, owned
// by the library so that a host binding (Julia ccall, Python ctypes) reuses the tuner.
//
// bm_plan_create times every candidate schedule -- CTA width {4, 8} warps x the
// wide/narrow split at {0, 8, 16, 24, 32, 48, 64, 96, all} band columns, as the host
// mirror's BandedBatch.tune does -- on a copy of the caller's batch with CUDA events,
// keeps the fastest, and stores its processing order (wide systems first, each part most
// expensive first) and the work-queue counters in device memory it allocates.  The
// choice is cached in the process per (device, batch shape), so a second plan for the
// same shape does not re-time.  bm_plan_execute_* then enqueue the scheduled batched
// solve with no allocation and no host synchronisation.  No counterpart in the
// reference (one system per call); per system they equal lu! + ldiv!
// (src/banded/BandedLU.jl:90-103, src/banded/linalg.jl:24-30) or the refined solve.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

struct bm_plan_st {
  int64_t count;
  int kind;  // 0: plain FP64 (bm_dgbsv_batched_sched), 1: refined (bm_dsgbsv_batched_sched)
  int device;
  bm_gb_schedule sched;
  int32_t* order;    // device, count entries
  int32_t* counter;  // device, 4 entries
  double best_ms;
  int candidates;
};

namespace bm {
namespace {

std::mutex g_plan_mu;
struct Choice {
  int64_t cols;  // systems with more band columns than this are wide
  int warps;
  double ms;
};
std::map<std::string, Choice> g_plan_cache;

double sys_cost(const bm_gb_desc& d) {
  return (double)d.n * (2.0 * d.kl * (d.kl + d.ku) + d.kl) + 2.0 * d.nrhs * d.n * (2.0 * d.kl + d.ku + 1);
}

// order (wide systems first, each part most expensive first) and the schedule bounds
void make_order(const bm_gb_desc* h, int64_t count, int64_t narrow_cols, int warps, std::vector<int32_t>& order,
                bm_gb_schedule& sc) {
  std::vector<int32_t> wide, narrow;
  for (int64_t s = 0; s < count; ++s) (h[s].kl + h[s].ku + 1 > narrow_cols ? wide : narrow).push_back((int32_t)s);
  auto by_cost = [&](int32_t a, int32_t b) {
    const double ca = sys_cost(h[a]), cb = sys_cost(h[b]);
    return ca > cb || (ca == cb && a < b);
  };
  std::stable_sort(wide.begin(), wide.end(), by_cost);
  std::stable_sort(narrow.begin(), narrow.end(), by_cost);
  order = wide;
  order.insert(order.end(), narrow.begin(), narrow.end());
  sc.n_wide = (int64_t)wide.size();
  sc.warps = warps;
  sc.wide_kl = sc.wide_ku = sc.narrow_kl = sc.narrow_ku = 0;
  for (int32_t s : wide) {
    sc.wide_kl = std::max(sc.wide_kl, h[s].kl);
    sc.wide_ku = std::max(sc.wide_ku, h[s].ku);
  }
  for (int32_t s : narrow) {
    sc.narrow_kl = std::max(sc.narrow_kl, h[s].kl);
    sc.narrow_ku = std::max(sc.narrow_ku, h[s].ku);
  }
}

std::string shape_key(int dev, int kind, const bm_gb_desc* h, int64_t count) {
  std::string k = std::to_string(dev) + ":" + std::to_string(kind) + ":";
  for (int64_t s = 0; s < count; ++s) {
    const int64_t f[4] = {h[s].n, h[s].kl, h[s].ku, h[s].nrhs};
    k.append(reinterpret_cast<const char*>(f), sizeof(f));
  }
  return k;
}

// Buffers of a timing run (the batch copied, plus the refined solve's workspace).
struct Scratch {
  double *AB = nullptr, *B = nullptr, *X = nullptr, *berr = nullptr;
  float *AB32 = nullptr, *R32 = nullptr;
  int64_t *ipiv = nullptr, *info = nullptr;
  int32_t* iters = nullptr;
  ~Scratch() {
    cudaFree(AB); cudaFree(B); cudaFree(X); cudaFree(berr); cudaFree(AB32); cudaFree(R32);
    cudaFree(ipiv); cudaFree(info); cudaFree(iters);
  }
};

}  // namespace
}  // namespace bm

// Arguments in order: plan 1, count 2, host_descs 3, descs 4, kind 5, AB 6, B 7.
extern "C" int bm_plan_create(bm_plan* plan, int64_t count, const bm_gb_desc* host_descs, const bm_gb_desc* descs,
                              int kind, const double* AB, const double* B, bm_stream_t stream) {
  using namespace bm;
  if (!plan) return -1;
  *plan = nullptr;
  if (count <= 0 || count > 0x7fffffff) return -2;
  if (!host_descs) return -3;
  if (!descs) return -4;
  if (kind != 0 && kind != 1) return -5;
  if (!AB) return -6;
  if (!B) return -7;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const char* name = "bm_plan_create";
  int dev = 0;
  int r = cuda_status(cudaGetDevice(&dev), name);
  if (r) return r;
  int64_t ab_len = 0, b_len = 0, piv_len = 0, max_cols = 1;
  for (int64_t q = 0; q < count; ++q) {
    const bm_gb_desc& d = host_descs[q];
    ab_len = std::max(ab_len, d.ab_offset + d.ldab * d.n);
    b_len = std::max(b_len, d.b_offset + d.ldb * std::max<int64_t>(d.nrhs - 1, 0) + d.n);
    piv_len = std::max(piv_len, d.ipiv_offset + d.n);
    max_cols = std::max(max_cols, d.kl + d.ku + 1);
  }
  bm_plan_st* p = new bm_plan_st();
  p->count = count;
  p->kind = kind;
  p->device = dev;
  p->order = nullptr;
  p->counter = nullptr;
  p->best_ms = -1.0;
  p->candidates = 0;
  auto fail = [&](int code) {
    cudaFree(p->order);
    cudaFree(p->counter);
    delete p;
    return code;
  };
  if ((r = cuda_status(cudaMalloc(&p->order, count * sizeof(int32_t)), name))) return fail(r == BM_ERR_CUDA ? BM_ERR_NOMEM : r);
  if ((r = cuda_status(cudaMalloc(&p->counter, 4 * sizeof(int32_t)), name))) return fail(BM_ERR_NOMEM);
  const std::string key = shape_key(dev, kind, host_descs, count);
  bool cached = false;
  Choice choice{0, 4, -1.0};
  {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    auto it = g_plan_cache.find(key);
    if (it != g_plan_cache.end()) {
      choice = it->second;
      cached = true;
    }
  }
  std::vector<int32_t> order;
  if (!cached) {
    Scratch sc;
    if (cudaMalloc(&sc.AB, ab_len * 8) || cudaMalloc(&sc.B, b_len * 8) || cudaMalloc(&sc.ipiv, piv_len * 8) ||
        cudaMalloc(&sc.info, count * 8)) {
      set_error("%s: no device memory for the timing runs", name);
      return fail(BM_ERR_NOMEM);
    }
    if (kind == 1 && (cudaMalloc(&sc.X, b_len * 8) || cudaMalloc(&sc.AB32, ab_len * 4) ||
                      cudaMalloc(&sc.R32, b_len * 4) || cudaMalloc(&sc.iters, count * 4) ||
                      cudaMalloc(&sc.berr, count * 8))) {
      set_error("%s: no device memory for the timing runs", name);
      return fail(BM_ERR_NOMEM);
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int64_t cols_list[] = {0, 8, 16, 24, 32, 48, 64, 96, int64_t(1) << 30};
    double best = 1e300;
    for (int warps : {4, 8}) {
      std::vector<int64_t> widths;
      for (int64_t c : cols_list) widths.push_back(std::min(c, max_cols));
      std::sort(widths.begin(), widths.end());
      widths.erase(std::unique(widths.begin(), widths.end()), widths.end());
      for (int64_t cols : widths) {
        bm_gb_schedule sched;
        make_order(host_descs, count, cols, warps, order, sched);
        if ((r = cuda_status(cudaMemcpyAsync(p->order, order.data(), count * 4, cudaMemcpyHostToDevice, s), name)))
          break;
        float best_rep = 1e30f;
        bool ok = true;
        for (int rep = 0; rep < 2 && ok; ++rep) {  // the first run warms up, the second is timed
          cudaMemcpyAsync(sc.AB, AB, ab_len * 8, cudaMemcpyDeviceToDevice, s);
          cudaMemcpyAsync(sc.B, B, b_len * 8, cudaMemcpyDeviceToDevice, s);
          cudaEventRecord(e0, s);
          int st = kind == 0 ? bm_dgbsv_batched_sched(count, descs, p->order, &sched, sc.AB, sc.ipiv, sc.B, sc.info,
                                                      p->counter, stream)
                             : bm_dsgbsv_batched_sched(count, descs, p->order, &sched, sc.AB, sc.B, sc.X, sc.ipiv,
                                                       sc.info, sc.AB32, sc.R32, sc.iters, sc.berr, p->counter, 1e-10,
                                                       30, stream);
          cudaEventRecord(e1, s);
          if (st != BM_OK) {  // this schedule's shared memory does not fit: skip it
            ok = false;
            break;
          }
          if (cudaEventSynchronize(e1) != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            set_error("%s: a timing run failed: %s", name, cudaGetErrorString(cudaGetLastError()));
            return fail(BM_ERR_CUDA);
          }
          float ms = 0.f;
          cudaEventElapsedTime(&ms, e0, e1);
          if (rep == 1) best_rep = ms;
        }
        if (!ok) continue;
        ++p->candidates;
        if (best_rep < best) {
          best = best_rep;
          choice = Choice{cols, warps, (double)best_rep};
        }
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best >= 1e300) {
      set_error("%s: no candidate schedule fits this batch", name);
      return fail(BM_ERR_UNSUPPORTED);
    }
    std::lock_guard<std::mutex> lk(g_plan_mu);
    g_plan_cache[key] = choice;
  }
  // the chosen schedule and its order, for the executions
  p->best_ms = choice.ms;
  make_order(host_descs, count, choice.cols, choice.warps, order, p->sched);
  if ((r = cuda_status(cudaMemcpyAsync(p->order, order.data(), count * 4, cudaMemcpyHostToDevice, s), name)))
    return fail(r);
  if ((r = cuda_status(cudaStreamSynchronize(s), name))) return fail(r);
  *plan = p;
  return BM_OK;
}

extern "C" int bm_plan_destroy(bm_plan plan) {
  if (!plan) return -1;
  cudaFree(plan->order);
  cudaFree(plan->counter);
  delete plan;
  return BM_OK;
}

extern "C" int bm_plan_schedule(bm_plan plan, bm_gb_schedule* sched, double* tuned_ms, int64_t* candidates) {
  if (!plan) return -1;
  if (!sched) return -2;
  *sched = plan->sched;
  if (tuned_ms) *tuned_ms = plan->best_ms;
  if (candidates) *candidates = plan->candidates;
  return BM_OK;
}

extern "C" int bm_plan_execute_dgbsv(bm_plan plan, const bm_gb_desc* descs, double* AB, int64_t* ipiv, double* B,
                                     int64_t* info, bm_stream_t stream) {
  if (!plan || plan->kind != 0) return -1;
  return bm_dgbsv_batched_sched(plan->count, descs, plan->order, &plan->sched, AB, ipiv, B, info, plan->counter,
                                stream);
}

extern "C" int bm_plan_execute_dsgbsv(bm_plan plan, const bm_gb_desc* descs, const double* AB, const double* B,
                                      double* X, int64_t* ipiv, int64_t* info, float* AB32, float* R32,
                                      int32_t* iters, double* berr, double tol, int64_t maxit, bm_stream_t stream) {
  if (!plan || plan->kind != 1) return -1;
  return bm_dsgbsv_batched_sched(plan->count, descs, plan->order, &plan->sched, AB, B, X, ipiv, info, AB32, R32,
                                 iters, berr, plan->counter, tol, maxit, stream);
}
