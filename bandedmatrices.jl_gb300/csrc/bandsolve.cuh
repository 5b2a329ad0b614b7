// FP32 banded triangular sweeps of gbtrs 'N' for ONE right-hand side per CTA, fed by
// 1-D TMA bulk copies: the correction solves of the single-system refined solve
// (dsgbsv.cu).  Same arithmetic as dgbtrs 'N' in FP32: forward -- interchange
// b(j) <-> b(ipiv(j)), then b(j+1 .. j+lm) -= L(:, j) b(j); backward -- x(j) = b(j) *
// (1/U(j,j)), then b(j-kv .. j-1) -= U(:, j) x(j).
//
// A sweep is a chain of n dependent steps, so its speed is the latency of one step.
// The steps are taken in chunks of 32 by a CTA of kBsWarps warps:
//   * warp 0 holds the chunk's 32 rows in registers (lane i: position 32c + i, where a
//     position is the row for the forward sweep and n-1-row for the backward one) and
//     takes the 32 steps one after another, updating only those rows -- one shuffle
//     and one fma per step on the critical path;
//   * the other warps apply the chunk's deferred updates to the rows further on (a
//     window of positions in shared memory), while warp 0 already solves the next
//     chunk; warp 0 itself applies them to the next chunk's 32 rows first.
// One CTA barrier per chunk separates the two.  Every row receives the updates of
// the steps in step order, so the result is gbtrs' order except where a pivot row
// lies beyond the chunk: its value is then brought up to date with the chunk's
// earlier steps by a warp reduction, and the row swapped into its place is stored
// pre-compensated for the same deferred terms (rare in practice: 0.8% of the steps of
// a randn + 16 I band with l = u = 128).
// The 32 factor columns a chunk needs are consecutive in the FP32 gbtrf storage, so one
// TMA bulk copy brings the whole block (32 x ldf floats) into a ring of `stages`
// slots, issued stages-1 chunks ahead and completed on an mbarrier per slot.  One large
// copy per chunk keeps a single SM's load stream at TMA speed; per-column copies
// (bulk or cp.async, bounded by the SM's outstanding-request limit) measured ~19 GB/s,
// which set the step time.  The factor storage's leading dimension must be a multiple
// of 4 and its base 16-byte aligned.  Every wait is bounded; on expiry the status word
// is set and the sweep stops after its issued copies have landed (bounded again).
#pragma once
#include "common.cuh"

namespace bm {

constexpr int kBsWarps = 4;    // warp 0 solves, warps 1.. update
constexpr int kBsWin = 512;    // window of positions (power of two >= band + 96)
constexpr int kBsMaxBand = kBsWin - 96;

// Shared memory of a sweep CTA: [0, 64) the mbarriers (two sweeps x up to 4 slots),
// [128, 144) the updaters' progress, [256, 512) x of the last two chunks, [512, 2560)
// the window, then the ring of `stages` slots of 32 x ldf floats: 4 slots where they
// fit in 227 KB, else 3.
constexpr int kBsRingOff = 512 + kBsWin * 4;
__host__ __device__ inline int bs_stages(i64 ldf) { return kBsRingOff + 4 * 128 * ldf <= 227 * 1024 ? 4 : 3; }
__host__ __device__ inline int bs_smem_bytes(i64 ldf) { return kBsRingOff + bs_stages(ldf) * 128 * (int)ldf; }

// A forward step's interchange of row t with its pivot row p (window-relative, p > t).
// Inside the chunk (p < 32) the two lanes exchange.  Beyond it, row p is in the window:
// wait until the updaters' deferred updates of chunk c-1 reached the window, bring row p
// up to date with this chunk's steps before t (a warp sum of L(p, j_t') x_t'), and
// store row t's value there pre-compensated for the same terms, which the updaters
// subtract later.  Rare (about 1.5% of the steps of the benchmark band); not inlined, so
// the unrolled steps stay small.  Returns the lane's new value, the step's x and
// whether the wait held.
struct BsSwap {
  float v, x;
  bool ok;
};
static __device__ __noinline__ BsSwap bs_swap(float v, float x, int t, int p, i64 c, const float* col0, int cs,
                                              int kv, int seg0, int kl, float* win, volatile int* done) {
  const int lane = threadIdx.x & 31;
  BsSwap r;
  r.ok = true;
  if (p < 32) {
    const float vp = __shfl_sync(0xffffffffu, v, p);
    r.v = lane == p ? x : lane == t ? vp : v;
    r.x = vp;
    return r;
  }
  bool ready = false;
  for (uint32_t it = 0; it < kSpinLimit && !ready; ++it) {
    ready = true;
    for (int w = 1; w < kBsWarps; ++w) ready = ready && done[w] >= c - 1;
  }
  __threadfence_block();
  const int dq = p - lane;
  float term = (lane < t && dq <= kl) ? col0[lane * cs + kv + dq - seg0] * v : 0.0f;
#pragma unroll
  for (int o = 16; o; o >>= 1) term += __shfl_xor_sync(0xffffffffu, term, o);
  float* wp = win + ((32 * c + p) & (kBsWin - 1));
  const float cur = *wp - term;
  __syncwarp();
  if (lane == 0) *wp = x + term;
  r.v = lane == t ? cur : v;
  r.x = cur;
  r.ok = ready;
  return r;
}

// One sweep of the right-hand side b (length n) by the whole CTA (kBsWarps warps).
// FWD: chunk c holds steps j = 32c + t (t < 32, j < n - 1); backward: steps
// j = n-1 - 32c - t (j >= 0).  Step j reads its column of the factor storage F: FWD the
// multipliers (rows kv+1 .. kv+kl), backward U above the diagonal and the diagonal (row
// kv).  bars: this sweep's `stages` mbarriers, initialised with one arrival.  Returns
// false (for every thread) if a wait ran out.
template <bool FWD>
__device__ bool bs_sweep(i64 n, int kl, int ku, const float* __restrict__ F, i64 ldf, const i64* __restrict__ ipiv,
                         float* __restrict__ b, unsigned char* smem, uint64_t* bars, int stages, int* status) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int kv = kl + ku;
  const int seg0 = FWD ? kv + 1 : 0;  // the rows read start here (column offsets relative to it)
  const int KB = FWD ? kl : kv;  // reach of a step
  const int KBe = KB > 32 ? KB : 32;  // the window is filled this far beyond the chunk (>= the next chunk)
  const i64 nsteps = FWD ? n - 1 : n;
  volatile int* done = reinterpret_cast<volatile int*>(smem + 128);  // [kBsWarps]: last chunk updated
  float* xbuf = reinterpret_cast<float*>(smem + 256);  // [2][32]
  float* win = reinterpret_cast<float*>(smem + 512);
  float* ring = reinterpret_cast<float*>(smem + kBsRingOff);
  if (nsteps <= 0) return true;
  const i64 nchunks = (nsteps + 31) / 32;
  auto pos_row = [&](i64 s) -> i64 { return FWD ? s : n - 1 - s; };
  auto load_pos = [&](i64 s) -> float { return s < n ? b[pos_row(s)] : 0.0f; };
  auto winp = [&](i64 s) -> float& { return win[s & (kBsWin - 1)]; };
  const int S = stages;
  const int lds = (int)ldf;
  auto cols_of = [&](i64 c) -> int { return (int)min((i64)32, nsteps - 32 * c); };
  // the chunk's block: columns 32c .. (FWD) or n-32c-cols .. n-1-32c (backward)
  auto issue = [&](i64 c) {  // by one thread
    if (c >= nchunks) return;
    const int st = (int)(c % S), cols = cols_of(c);
    const i64 first = FWD ? 32 * c : n - 32 * c - cols;
    const uint32_t bytes = (uint32_t)(cols * lds * 4);
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&bars[st], bytes);
    bulk_g2s(ring + (i64)st * 32 * lds, F + first * ldf, bytes, &bars[st]);
  };
  auto wait_chunk = [&](i64 c) -> bool { return mbar_wait(&bars[c % S], (uint32_t)((c / S) & 1)); };
  // column of step t of chunk c in its slot (plus seg0), and the stride between steps
  auto col_base = [&](i64 c) -> const float* {
    const float* slot = ring + (c % S) * 32 * lds;
    return FWD ? slot + seg0 : slot + (cols_of(c) - 1) * lds;
  };
  const int cs = FWD ? lds : -lds;
  auto load_piv = [&](i64 c) -> i64 {  // window-relative pivot of step lane of chunk c (FWD)
    const i64 j = 32 * c + lane;
    return (FWD && j < nsteps) ? ipiv[j] - 1 - 32 * c : lane;
  };

  // ---- set-up: chunk 0's rows in warp 0, the positions chunk 0 reaches in the window
  float v = 0.0f;
  i64 pv_cur = 0, pv_next = 0;
  if (warp == 0) {
    v = load_pos(lane);
    if (FWD) {
      pv_cur = load_piv(0);
      pv_next = load_piv(1);
    }
  }
  for (int q = tid; q < KBe; q += 32 * kBsWarps) winp(32 + q) = load_pos(32 + q);
  if (tid < kBsWarps) done[tid] = -1;
  if (tid == 32)
    for (int c0 = 0; c0 < S - 1; ++c0) issue(c0);
  __syncthreads();

  bool failed = false;  // this thread's wait ran out; the CTA leaves together (barrier OR)
  i64 c = 0;
  for (; c < nchunks; ++c) {
    const int cols = (int)min((i64)32, nsteps - 32 * c);
    const int remi = (int)min(n - 1 - 32 * c, (i64)1 << 30);
    const float* col0 = col_base(c);
    // ---- warp 0: the chunk's steps
    if (warp == 0) {
      if (!wait_chunk(c)) {
        failed = true;
      } else {
        const int pvl = (int)pv_cur;
        float rc = 0.0f;
        if (!FWD) rc = lane < cols ? __frcp_rn(col0[lane * cs + kv]) : 0.0f;
        // steps that interchange (pivot row != own row), one bit per step
        const unsigned swaps = FWD ? __ballot_sync(0xffffffffu, lane < cols && pvl != lane) : 0u;
        // one step: x(j) to every lane, the interchange if any, then the chunk's rows below
        auto step = [&](int t, int lim) {
          float x;
          if (FWD) {
            x = __shfl_sync(0xffffffffu, v, t);
            if ((swaps >> t) & 1u) {  // warp-uniform
              const BsSwap r = bs_swap(v, x, t, __shfl_sync(0xffffffffu, pvl, t), c, col0, cs, kv, seg0, kl, win, done);
              v = r.v;
              x = r.x;
              failed = failed || !r.ok;
            }
          } else {
            x = __shfl_sync(0xffffffffu, v * rc, t);
            if (lane == t) v = x;
          }
          const int d = lane - t;
          if (d >= 1 && d <= lim) v = fmaf(-col0[t * cs + (FWD ? kv + d - seg0 : kv - d)], x, v);
        };
        if (cols == 32 && remi >= KB + 31 && swaps == 0u) {
          // a full chunk without interchanges (every backward chunk, most forward ones):
          // every step reaches KB rows
#pragma unroll
          for (int t = 0; t < 32; ++t) {
            const float x = __shfl_sync(0xffffffffu, FWD ? v : v * rc, t);
            if (!FWD && lane == t) v = x;
            const int d = lane - t;
            if (d >= 1 && d <= KB) v = fmaf(-col0[t * cs + (FWD ? kv + d - seg0 : kv - d)], x, v);
          }
        } else if (FWD && cols == 32 && remi >= KB + 31) {
          // a full forward chunk with interchanges: by quarters of 8 steps, the quarters
          // without one unrolled (most of them), the others through the general step
          for (int q = 0; q < 4; ++q) {
            const int t0 = 8 * q;
            if (((swaps >> t0) & 0xffu) == 0u) {
#pragma unroll
              for (int k = 0; k < 8; ++k) {
                const int t = t0 + k;
                const float x = __shfl_sync(0xffffffffu, v, t);
                const int d = lane - t;
                if (d >= 1 && d <= KB) v = fmaf(-col0[t * cs + (kv + d - seg0)], x, v);
              }
            } else {
#pragma unroll 1
              for (int k = 0; k < 8; ++k) step(t0 + k, KB);
            }
          }
        } else {
#pragma unroll 4
          for (int t = 0; t < cols; ++t) step(t, min(KB, remi - t));
        }
        xbuf[(c & 1) * 32 + lane] = v;
        const i64 s = 32 * c + lane;
        if (s < n) b[pos_row(s)] = v;
      }
    }
    if (__syncthreads_or(failed)) break;
    const float* xc = xbuf + (c & 1) * 32;
    if (warp == 0) {
      // ---- the chunk's updates of the next chunk's rows
      float w = winp(32 * (c + 1) + lane);
      auto upd = [&](int t, int lim) {
        const float x = __shfl_sync(0xffffffffu, v, t);  // every lane takes part in the shuffle
        const int d = 32 + lane - t;
        if (d <= lim) w = fmaf(-col0[t * cs + (FWD ? kv + d - seg0 : kv - d)], x, w);
      };
      if (cols == 32 && remi >= KB + 31) {
#pragma unroll
        for (int t = 0; t < 32; ++t) upd(t, KB);
      } else {
#pragma unroll 1
        for (int t = 0; t < cols; ++t) upd(t, min(KB, remi - t));
      }
      v = w;
      if (FWD) {
        pv_cur = pv_next;
        pv_next = load_piv(c + 2);
      }
    } else {
      // ---- updaters: the chunk's updates of the positions beyond the next chunk
      if (tid == 32) issue(c + S - 1);  // into the slot of chunk c-1, whose readers are done
      if (!wait_chunk(c)) failed = true;  // (landed: warp 0 waited for it)
      float enter = 0.0f;
      const i64 s_in = 32 * c + 32 + KBe + lane;  // positions that enter the window
      if (warp == 1) enter = load_pos(s_in);
      const i64 p1 = min(32 * c + 31 + KB, n - 1);
      for (int db = 64 + (tid - 32); 32 * c + db <= p1; db += 32 * (kBsWarps - 1)) {
        // position 32c + db; step t reaches it at d = db - t >= 33
        float& wr = winp(32 * c + db);
        float w = wr;
        const float* cp = col0 + (FWD ? kv + db - seg0 : kv - db);  // + t (cs -+ 1)
#pragma unroll 8
        for (int t = 0; t < cols; ++t)
          if (db - t <= KB) w = fmaf(-cp[t * (FWD ? cs - 1 : cs + 1)], xc[t], w);
        wr = w;
      }
      if (warp == 1) winp(s_in) = enter;
      __syncwarp();
      if (lane == 0) {
        __threadfence_block();
        done[warp] = (int)c;
      }
    }
  }
  const bool ok = !__syncthreads_or(failed);
  if (!ok && tid == 0) record_status(status, BM_STATUS_TIMEOUT);
  if (ok) {
    if (FWD && warp == 0) {  // row n-1 takes no step of its own; it may be the chunk after the last
      const i64 s = 32 * nchunks + lane;
      if (s == n - 1) b[pos_row(s)] = v;
    }
  } else if (tid == 32) {  // let the copies already issued land before the shared memory is reused
    for (i64 c2 = c > 0 ? c - 1 : 0; c2 < min(nchunks, c + S - 1); ++c2) (void)wait_chunk(c2);
  }
  __syncthreads();
  return ok;
}

}  // namespace bm
