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

// ------------------------------------------------------------------ tiny bands
// Bands with kl >= 1 and kl * (kl + ku + 1) <= 32 (the (4,3) band fills 32 lanes).  On
// GB300 an FP64 instruction holds its warp for about 64 cycles and a division for about
// 570, so a step should issue as few of them as possible, each over the whole window.
// One warp; lane L = c*kl + (r-1) holds the window element (row j+r, column j+c),
// r = 1..kl, c = 0..kv, and a copy of the element of the window's row 0 in its column
// (row j, column j+c).  A dgbtf2 step is then:
//   * idamax over column 0 (a warp argmax, first index on ties; the pivot key of row 0
//     from the copy);
//   * the interchange of rows 0 and jp in every column: one shuffle within the column;
//   * U's row j (the copies, after the interchange) and column j's multipliers
//     (rcp * a on the column-0 lanes, rcp = 1 / pivot) go to memory;
//   * the rank-1 update of the other columns: one fma per lane, skipped where U(j, .)
//     is zero;
//   * the slide of the window: (r, c) <- (r+1, c+1) by shuffle, the entering row
//     (prefetched kTinyPre steps ahead) into row kl, zeros (fill) into the new column.
// Each element receives dgbtf2's operations in dgbtf2's order: factors, pivots and info
// equal the unblocked result bit for bit.
constexpr int kTinyPre = 4;

template <typename T>
__global__ void __launch_bounds__(32) gbtrf_tiny_kernel(i64 m, i64 n, int kl, int ku, T* ab, i64 ldab, i64* ipiv,
                                                        i64* info) {
  const int lane = threadIdx.x, kv = kl + ku;
  const i64 mn = min(m, n);
  const int c = lane / kl, r = lane - c * kl + 1;
  const bool act = c <= kv;
  // element (i, col) of the original band, zero outside it and outside the matrix
  // (the fill rows of the storage are workspace on entry, as in dgbtrf)
  auto elem = [&](i64 i, i64 col) -> T {
    const i64 d = i - col;
    return (i < m && col < n && d >= -ku && d <= kl) ? ab[(kv + d) + col * ldab] : T(0);
  };
  T a = act ? elem(r, c) : T(0);
  T u = act ? elem(0, c) : T(0);
  const bool enter = act && r == kl;  // lanes of the window's last row
  T e[kTinyPre];                       // e[s]: row j+s+1+kl of column j+s+1+c, at step j
#pragma unroll
  for (int s = 0; s < kTinyPre; ++s) e[s] = enter ? elem(s + 1 + kl, s + 1 + c) : T(0);
  const int src_next = min((c + 1) * kl + r, 31), src_row1 = min((c + 1) * kl, 31);
  i64 inf = 0;
  // one step on ring slot `ent`: its value enters at the slide, and the slot is then
  // reloaded for step j + kTinyPre (a slot is only read at its own step, so no
  // instruction waits on a load in flight)
  auto step = [&](i64 j, T& ent) {
    const int km = (int)min((i64)kl, m - 1 - j);
    unsigned long long key = 0ull;
    int idx = 0x7fffffff;
    if (c == 0) {
      if (r == 1) {
        key = pivot_key(u, true);
        idx = 0;
      }
      if (r <= km) {
        const unsigned long long k = pivot_key(a, false);
        if (idx == 0x7fffffff || k > key) {
          key = k;
          idx = r;
        }
      }
    }
    const int jp = warp_argmax_first(key, idx);
    const T piv = __shfl_sync(0xffffffffu, jp == 0 ? u : a, jp == 0 ? 0 : jp - 1);
    const bool ns = is_nonzero(piv);
    if (lane == 0) ipiv[j] = j + jp + 1;
    if (ns) {
      const T rcp = T(1) / piv;
      if (jp != 0) {  // rows 0 and jp trade places in every column
        const T t = __shfl_sync(0xffffffffu, a, min(c * kl + jp - 1, 31));
        if (r == jp) a = u;
        u = t;
      }
      if (c == 0 && r <= km) a = rcp * a;  // the multipliers
    } else if (inf == 0) {
      inf = j + 1;
    }
    if (act && r == 1 && j + c < n) ab[(kv - c) + (j + c) * ldab] = u;  // U(j, j+c)
    if (c == 0 && r <= km) ab[(kv + r) + j * ldab] = a;                 // column j below the diagonal
    if (ns) {
      const T l = __shfl_sync(0xffffffffu, a, r - 1);  // the multiplier of row j+r
      if (act && c >= 1 && r <= km && is_nonzero(u)) a = fma(l, -u, a);
    }
    // slide to step j+1
    const T na = __shfl_sync(0xffffffffu, a, src_next);
    const T nu = __shfl_sync(0xffffffffu, a, src_row1);
    const bool inside = c + 1 <= kv;
    a = r < kl ? (inside ? na : T(0)) : ent;
    u = inside ? nu : T(0);
    ent = enter ? elem(j + kTinyPre + 1 + kl, j + kTinyPre + 1 + c) : T(0);
  };
  for (i64 j = 0; j < mn; j += kTinyPre) {
#pragma unroll
    for (int s = 0; s < kTinyPre; ++s)
      if (j + s < mn) step(j + s, e[s]);
  }
  // m < n: the fill rows of columns mn+ku+1 .. mn+kv-1 at rows >= mn (no step reaches them)
  for (i64 cc = mn + ku + 1 + lane; cc < min(mn + kv, n); cc += 32)
    for (i64 i = max(mn, cc - kv); i <= cc - ku - 1; ++i) ab[(kv + i - cc) + cc * ldab] = T(0);
  if (lane == 0) *info = inf;
}

template <typename T>
int gbtrf_tiny_run(i64 m, i64 n, i64 kl, i64 ku, T* ab, i64 ldab, i64* ipiv, i64* info, cudaStream_t stream,
                   const char* name) {
  if (!tiny_fits(kl, ku)) {
    set_error("%s: band (%lld, %lld) outside the tiny-band kernel", name, (long long)kl, (long long)ku);
    return BM_ERR_UNSUPPORTED;
  }
  gbtrf_tiny_kernel<T><<<1, 32, 0, stream>>>(m, n, (int)kl, (int)ku, ab, ldab, ipiv, info);
  return launch_status(name);
}

// gbtrs 'N' for tiny bands, one warp per right-hand side.
//   forward (dgbtrs: interchange, then b(j+1:j+lm) -= b(j) * l, skipped when b(j) == 0):
//     lane r holds b(j+r), r = 0..kl; the interchange is a shuffle, the update one fma;
//   backward (dtbsv 'U','N','N'): lane p holds x(j-p), p = 0..kv; x(j) /= U(j, j) through
//     the staged reciprocal pair of U(j, j) (taken for 32 steps at a time, one per lane,
//     off the critical path), then x(j-p) -= x(j) * U(j-p, j), skipped when x(j) == 0.
// The L and U columns and the entering b rows are loaded kTinyPre steps ahead.
template <typename T>
__global__ void __launch_bounds__(32) gbtrs_tiny_kernel(i64 n, int kl, int ku, i64 nrhs, const T* __restrict__ ab,
                                                        i64 ldab, const i64* __restrict__ ipiv, T* B, i64 ldb) {
  const int lane = threadIdx.x, kv = kl + ku;
  for (i64 rhs = blockIdx.x; rhs < nrhs; rhs += gridDim.x) {
    T* b = B + rhs * ldb;
    if (kl > 0 && n > 1) {
      const bool act = lane <= kl;
      T x = (act && lane < n) ? b[lane] : T(0);
      // ring slot s holds, for its step j: lv = L(j+lane, j) (lanes 1..kl), pv = ipiv(j),
      // ev = b(j+1+kl); a slot is read at its own step only, then reloaded kTinyPre ahead
      T lv[kTinyPre], ev[kTinyPre];
      i64 pv[kTinyPre];
      auto fetch = [&](i64 j, T& l_, i64& p_, T& e_) {
        const bool ok = j < n - 1;
        l_ = (ok && lane >= 1 && lane <= kl && j + lane < n) ? ab[(kv + lane) + j * ldab] : T(0);
        p_ = ok ? ipiv[j] : j + 1;
        e_ = (ok && lane == kl && j + 1 + kl < n) ? b[j + 1 + kl] : T(0);
      };
#pragma unroll
      for (int s = 0; s < kTinyPre; ++s) fetch(s, lv[s], pv[s], ev[s]);
      auto step = [&](i64 j, T& l_, i64& p_, T& e_) {
        const int jp = (int)(p_ - 1 - j);
        const int lm = (int)min((i64)kl, n - 1 - j);
        if (jp != 0) {
          const T t = __shfl_sync(0xffffffffu, x, jp);
          const T x0 = __shfl_sync(0xffffffffu, x, 0);
          if (lane == 0) x = t;
          if (lane == jp) x = x0;
        }
        if (lane == 0) b[j] = x;  // b(j) is final
        const T bj = __shfl_sync(0xffffffffu, x, 0);
        if (is_nonzero(bj) && lane >= 1 && lane <= lm) x = fma(l_, -bj, x);
        const T nx = __shfl_sync(0xffffffffu, x, min(lane + 1, 31));
        x = lane < kl ? nx : e_;
        fetch(j + kTinyPre, l_, p_, e_);
      };
      for (i64 j = 0; j < n - 1; j += kTinyPre) {
#pragma unroll
        for (int s = 0; s < kTinyPre; ++s)
          if (j + s < n - 1) step(j + s, lv[s], pv[s], ev[s]);
      }
      // the last row of the window is final
      if (lane == 0) b[n - 1] = x;
    }
    __syncwarp();
    {
      const bool act = lane <= kv;
      T x = (act && n - 1 - lane >= 0) ? b[n - 1 - lane] : T(0);
      // ring slot s, for its step j: uv = U(j-lane, j) (lanes 0..kv; lane 0: U(j, j)),
      // ev = b(j-1-kv)
      T uv[kTinyPre], ev[kTinyPre];
      auto fetch = [&](i64 j, T& u_, T& e_) {
        u_ = (j >= 0 && act && j - lane >= 0) ? ab[(kv - lane) + j * ldab] : T(0);
        e_ = (j >= 0 && lane == kv && j - 1 - kv >= 0) ? b[j - 1 - kv] : T(0);
      };
#pragma unroll
      for (int s = 0; s < kTinyPre; ++s) fetch(n - 1 - s, uv[s], ev[s]);
      // the reciprocal pairs of U's diagonal, 32 steps at a time (lane k: step j0 - k);
      // the next block's diagonal is loaded a block ahead
      T yh = T(0), yl = T(0);
      T dnext = (n - 1 - lane >= 0) ? ab[kv + (n - 1 - lane) * ldab] : T(1);
      auto step = [&](i64 j, T& u_, T& e_) {
        const int k = (int)((n - 1 - j) & 31);
        if (k == 0) {
          div_rcp(dnext, yh, yl);
          dnext = (j - 32 - lane >= 0) ? ab[kv + (j - 32 - lane) * ldab] : T(1);
        }
        const T d = __shfl_sync(0xffffffffu, u_, 0);  // U(j, j)
        const T h = __shfl_sync(0xffffffffu, yh, k), lo = __shfl_sync(0xffffffffu, yl, k);
        T xj = __shfl_sync(0xffffffffu, x, 0);
        if (is_nonzero(xj)) {
          xj = div_staged(xj, d, h, lo);
          if (lane == 0) x = xj;
          if (lane >= 1 && act && j - lane >= 0) x = fma(-xj, u_, x);
        }
        if (lane == 0) b[j] = x;  // x(j) is final
        const T nx = __shfl_sync(0xffffffffu, x, min(lane + 1, 31));
        x = lane < kv ? nx : e_;
        fetch(j - kTinyPre, u_, e_);
      };
      for (i64 j = n - 1; j >= 0; j -= kTinyPre) {
#pragma unroll
        for (int s = 0; s < kTinyPre; ++s)
          if (j - s >= 0) step(j - s, uv[s], ev[s]);
      }
    }
    __syncwarp();
  }
}

template <typename T>
int gbtrs_tiny_run(i64 n, i64 kl, i64 ku, i64 nrhs, const T* ab, i64 ldab, const i64* ipiv, T* B, i64 ldb,
                   cudaStream_t stream, const char* name) {
  if (!tiny_solve_fits(kl, ku)) {
    set_error("%s: band (%lld, %lld) outside the tiny-band solve", name, (long long)kl, (long long)ku);
    return BM_ERR_UNSUPPORTED;
  }
  const unsigned grid = (unsigned)std::min<i64>(nrhs, (i64)num_sms() * 16);
  gbtrs_tiny_kernel<T><<<grid, 32, 0, stream>>>(n, (int)kl, (int)ku, nrhs, ab, ldab, ipiv, B, ldb);
  return launch_status(name);
}

template int gbtrf_tiny_run<float>(i64, i64, i64, i64, float*, i64, i64*, i64*, cudaStream_t, const char*);
template int gbtrf_tiny_run<double>(i64, i64, i64, i64, double*, i64, i64*, i64*, cudaStream_t, const char*);
template int gbtrs_tiny_run<float>(i64, i64, i64, i64, const float*, i64, const i64*, float*, i64, cudaStream_t,
                                   const char*);
template int gbtrs_tiny_run<double>(i64, i64, i64, i64, const double*, i64, const i64*, double*, i64, cudaStream_t,
                                    const char*);

template int gbtrs_reg_run<float>(i64, i64, i64, i64, const float*, i64, const i64*, float*, i64, cudaStream_t,
                                  const char*);
template int gbtrs_reg_run<double>(i64, i64, i64, i64, const double*, i64, const i64*, double*, i64, cudaStream_t,
                                   const char*);
template int gbtrf_reg_run<float>(i64, i64, i64, i64, float*, i64, i64*, i64*, cudaStream_t, const char*);
template int gbtrf_reg_run<double>(i64, i64, i64, i64, double*, i64, i64*, i64*, cudaStream_t, const char*);

}  // namespace bm
