// FP32 banded triangular sweeps of gbtrs 'N' for ONE system, one warp per right-hand
// side, fed by 1-D TMA bulk copies: the correction solves of the single-system refined
// solve (dsgbsv.cu).  Same arithmetic as dgbtrs 'N' in FP32: forward -- interchange
// b(j) <-> b(ipiv(j)), then b(j+1 .. j+lm) -= L(:, j) b(j); backward -- x(j) = b(j) *
// (1/U(j,j)), then b(j-kv .. j-1) -= U(:, j) x(j).
//
// The warp holds its window of b in registers: at a chunk of 32 steps starting at j0,
// slot s of lane i holds row j0 + 32 s + i (the backward sweep mirrors the index), so
// step t of the chunk reads row j from lane t, slot 0 -- a static register -- and the
// rows a step updates are lanes/slots at offsets d = 32 s + i - t.  After a chunk the
// slots shift down by one (the finished rows are stored, a new row enters slot NS-1).
// The factor columns a chunk needs are copied into a shared-memory ring of kBsStages
// chunks by bulk copies (one lane issues 32 per chunk, 2 chunks = 64 steps ahead, one
// mbarrier per stage); the factor storage's leading dimension must be a multiple of 4
// and its base 16-byte aligned so that every column segment is 16-byte aligned.
// Waits are bounded: on expiry the status word is set and the warp stops after its
// issued copies have landed (bounded again).
#pragma once
#include "common.cuh"

namespace bm {

constexpr int kBsStages = 3;

__host__ __device__ inline int bs_ns(int band) { return (band + 32 + 31) / 32; }
__host__ __device__ inline int bs_fwd_width(int kl, int ku) {  // floats per staged column (L part)
  const int kv = kl + ku;
  return ((kv + kl + 1 + 3) & ~3) - ((kv + 1) & ~3);
}
__host__ __device__ inline int bs_bwd_width(int kl, int ku) { return (kl + ku + 1 + 3) & ~3; }  // U part + diagonal
__host__ __device__ inline int bs_smem_bytes(int kl, int ku) {
  const int w = bs_fwd_width(kl, ku) > bs_bwd_width(kl, ku) ? bs_fwd_width(kl, ku) : bs_bwd_width(kl, ku);
  return 128 + kBsStages * 32 * w * 4;
}

template <int NS>
__device__ __forceinline__ float bs_get(const float (&v)[NS], int s) {
  float r = v[0];
#pragma unroll
  for (int k = 1; k < NS; ++k) r = s == k ? v[k] : r;
  return r;
}
template <int NS>
__device__ __forceinline__ void bs_set(float (&v)[NS], int s, float x) {
#pragma unroll
  for (int k = 0; k < NS; ++k)
    if (s == k) v[k] = x;
}

// One sweep.  FWD: chunk c covers steps j = 32c + t (t < 32, j < n - 1); backward: steps
// j = n-1 - 32c - t (j >= 0).  Column segment of step j in the factor storage F: FWD
// rows [seg0, seg0 + W) with seg0 = (kv+1) & ~3 (the multipliers at rows kv+1 ..
// kv+kl); backward rows [0, W) (U above the diagonal and the diagonal at row kv).
template <int NS, bool FWD>
__device__ bool bs_sweep(i64 n, int kl, int ku, const float* __restrict__ F, i64 ldf, const i64* __restrict__ ipiv,
                         float* __restrict__ b, float* ring, uint64_t* bars, int* status) {
  const int lane = threadIdx.x & 31;
  const int kv = kl + ku;
  const int seg0 = FWD ? ((kv + 1) & ~3) : 0;
  const int W = FWD ? bs_fwd_width(kl, ku) : bs_bwd_width(kl, ku);
  const i64 nsteps = FWD ? n - 1 : n;
  if (nsteps <= 0) return true;
  const i64 nchunks = (nsteps + 31) / 32;
  // row of lane `lane`, slot s at chunk c
  auto row_of = [&](i64 c, int s) -> i64 { return FWD ? 32 * (c + s) + lane : n - 1 - (32 * (c + s) + lane); };
  auto in_rows = [&](i64 r) { return r >= 0 && r < n; };
  auto step_j = [&](i64 c, int t) -> i64 { return FWD ? 32 * c + t : n - 1 - (32 * c + t); };
  auto issue = [&](i64 c) {
    if (lane != 0 || c >= nchunks) return;
    const int st = (int)(c % kBsStages);
    const int cols = (int)min((i64)32, nsteps - 32 * c);
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&bars[st], (uint32_t)(cols * W * 4));
    for (int q = 0; q < cols; ++q)
      bulk_g2s(ring + (st * 32 + q) * W, F + seg0 + step_j(c, q) * ldf, (uint32_t)(W * 4), &bars[st]);
  };
  float bw[NS];
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    const i64 r = row_of(0, s);
    bw[s] = in_rows(r) ? b[r] : 0.0f;
  }
  for (int c = 0; c < kBsStages - 1; ++c) issue(c);
  bool ok = true;
  i64 c = 0;
  for (; c < nchunks; ++c) {
    issue(c + kBsStages - 1);
    const int st = (int)(c % kBsStages);
    if (!mbar_wait(&bars[st], (uint32_t)((c / kBsStages) & 1))) {
      if (lane == 0) record_status(status, BM_STATUS_TIMEOUT);
      ok = false;
      break;
    }
    const float* col0 = ring + st * 32 * W;
    const i64 rn = row_of(c + NS, 0);  // the row entering slot NS-1 after this chunk
    const float nxt = in_rows(rn) ? b[rn] : 0.0f;
    i64 pv = 0;
    if (FWD) {
      const i64 j = 32 * c + lane;
      pv = j < nsteps ? ipiv[j] - 1 : j;
    }
    const int cols = (int)min((i64)32, nsteps - 32 * c);
    for (int t = 0; t < cols; ++t) {
      const i64 j = step_j(c, t);
      const float* colt = col0 + t * W;
      float x = __shfl_sync(0xffffffffu, bw[0], t);
      int lim;  // rows updated: offsets d = 1 .. lim
      if (FWD) {
        const i64 p = __shfl_sync(0xffffffffu, pv, t);
        if (p != j) {  // warp-uniform: the interchange with row p, inside the window
          const int dp = (int)(p - 32 * c), sp = dp >> 5, lp = dp & 31;
          const float vp = __shfl_sync(0xffffffffu, bs_get<NS>(bw, sp), lp);
          if (lane == lp) bs_set<NS>(bw, sp, x);
          if (lane == t) bw[0] = vp;
          x = vp;
        }
        lim = (int)min((i64)kl, n - 1 - j);
      } else {
        x = x * __frcp_rn(colt[kv]);
        if (lane == t) bw[0] = x;
        lim = (int)min((i64)kv, j);
      }
#pragma unroll
      for (int s = 0; s < NS; ++s) {
        const int d = 32 * s + lane - t;
        if (d >= 1 && d <= lim) bw[s] = fmaf(-colt[FWD ? kv + d - seg0 : kv - d], x, bw[s]);
      }
    }
    {  // the rows of slot 0 are final (in the last forward chunk, with row n-1)
      const i64 r = row_of(c, 0);
      if (in_rows(r)) b[r] = bw[0];
    }
#pragma unroll
    for (int s = 0; s < NS - 1; ++s) bw[s] = bw[s + 1];
    bw[NS - 1] = nxt;
    __syncwarp();
  }
  if (ok) {
    if (FWD) {  // row n-1 takes no step of its own; after a full last chunk it is in slot 0
      const i64 r = row_of(c, 0);
      if (r == n - 1) b[r] = bw[0];
    }
  } else {  // let the copies already issued land before the shared memory is released
    for (i64 c2 = c; c2 < min(nchunks, c + kBsStages); ++c2)
      (void)mbar_wait(&bars[c2 % kBsStages], (uint32_t)((c2 / kBsStages) & 1));
  }
  __syncwarp();
  return ok;
}

}  // namespace bm
