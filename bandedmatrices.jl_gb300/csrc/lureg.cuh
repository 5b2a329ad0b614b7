// Register-window banded LU (xGBTF2 semantics): one lane per window column.
//
// At step j the active part of the matrix is the window A(j:j+kl, j:j+kl+ku).  Lane t
// of a group of NL = 32*W lanes owns the columns c = t (mod NL); the column it owns at
// step j holds its rows j..j+kl in registers w[0..kl] (w[r] = A(j+r, c)).  A step is:
//   * the interchange: u = w[d], w[d] = w[0] (d = jp of the step, the same in every lane;
//     predicated selects, skipped when d == 0);
//   * U(j, c) = u goes to memory;
//   * the rank-1 update fused with the slide of the window:
//       w[r-1] = fma(l_r, -u, w[r])  (r = 1..KL; the plain shift w[r-1] = w[r] when
//     u == 0 or the pivot is zero, as dgbtf2 skips those columns);
//   * the row that enters the window (row j+1+kl, loaded kRegPre steps ahead) is placed
//     in w[kl].
// The lane of the next column then has that column's new rows; its warp transposes
// them through shared memory, finds the pivot (idamax: first index of the largest |a|),
// scales by the reciprocal of the pivot and publishes the step record (jp, a nonzero
// flag and the multipliers) for the next step, which the other lanes read after one
// group barrier.  Every element receives dgbtf2's operations in dgbtf2's order, so
// factors, pivots and info equal the oracle's bit for bit.
//
// Rows beyond kl in the register array (KL is a size class >= kl) and rows beyond the
// last row of the matrix hold values that are never read: the pivot search, the
// interchange and the stores touch rows 0..km only.
#pragma once
#include "lu.cuh"

namespace bm {

template <typename T>
struct RegVec;
template <>
struct RegVec<float> {
  using type = float4;
  static constexpr int n = 4;
  static __device__ __forceinline__ float get(const float4& v, int k) {
    return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
  }
};
template <>
struct RegVec<double> {
  using type = double2;
  static constexpr int n = 2;
  static __device__ __forceinline__ double get(const double2& v, int k) { return k == 0 ? v.x : v.y; }
};

// The register window: KL+1 values addressed with compile-time indices after
// unrolling.  Kept in 32-element pieces, which the compiler keeps in registers (one
// array of more than about 500 bytes is placed in local memory instead).
template <typename T, int N>
struct RegArr {
  static constexpr int sz(int k) { return N - 32 * k >= 32 ? 32 : (N - 32 * k > 0 ? N - 32 * k : 1); }
  T a0[sz(0)], a1[sz(1)], a2[sz(2)], a3[sz(3)], a4[sz(4)];
  __device__ __forceinline__ T& operator[](int p) {
    return p < 32 ? a0[p] : p < 64 ? a1[p - 32] : p < 96 ? a2[p - 64] : p < 128 ? a3[p - 96] : a4[p - 128];
  }
  __device__ __forceinline__ const T& operator[](int p) const {
    return p < 32 ? a0[p] : p < 64 ? a1[p - 32] : p < 96 ? a2[p - 64] : p < 128 ? a3[p - 96] : a4[p - 128];
  }
};

// The step record: jp, the nonzero-pivot flag and the multipliers of rows 1..KL
// (l[r-1]), 16-byte aligned for vector loads.
template <typename T, int KL>
struct __align__(16) RegStep {
  int d, ns, pad0, pad1;
  T l[KL];
};

// Entering rows are loaded kRegPre steps ahead through a per-lane ring.
constexpr int kRegPre = 8;

template <typename T, int KL, int NLMAX>
struct __align__(16) RegShared {
  RegStep<T, KL> rec[2];
  T scr[KL + 4];  // the pivot column, transposed from its lane's registers
  T pre[kRegPre * NLMAX];
  long long info;
};

// Size classes of the register window: 4, 8, 16, 32, then multiples of 16 up to 128.
// Class K holds the sizes (reg_cls_lo(K), K] ([0, 4] for K = 4).
constexpr int kRegMaxWarps = 8;
template <typename T>
__host__ __device__ constexpr int reg_kl_max() { return sizeof(T) == 4 ? 64 : 32; }
__host__ __device__ constexpr int reg_cls(long long x) {
  return x <= 4 ? 4 : x <= 8 ? 8 : x <= 16 ? 16 : x <= 32 ? 32 : (int)((x + 15) / 16 * 16);
}
__host__ __device__ constexpr int reg_cls_lo(int K) {
  return K == 4 ? 0 : K == 8 ? 5 : K == 16 ? 9 : K == 32 ? 17 : K - 15;
}
template <typename T>
__host__ __device__ inline int reg_class(long long kl, long long ku) {
  if (kl < 0 || ku < 0 || kl > reg_kl_max<T>() || kl + ku + 1 > 32 * kRegMaxWarps) return 0;
  return reg_cls(kl);
}
template <typename T>
__host__ __device__ inline int reg_kv_class(long long kv) {
  if (kv < 0 || kv > 2 * reg_kl_max<T>()) return 0;
  return reg_cls(kv);
}

// f(RegK<K>{}) for a class K <= KMAX (callers pass valid classes only).
template <int K>
struct RegK {
  static constexpr int v = K;
};
template <int KMAX, typename F>
__host__ __device__ inline auto reg_dispatch(int K, F&& f) {
#define BM_RK(k) \
  case k:        \
    if constexpr (k <= KMAX) return f(RegK<k>{});
  switch (K) {
    BM_RK(8) BM_RK(16) BM_RK(32) BM_RK(48) BM_RK(64) BM_RK(80) BM_RK(96) BM_RK(112) BM_RK(128)
    default:
      break;
  }
#undef BM_RK
  return f(RegK<4>{});
}

__host__ __device__ inline int reg_warps(long long kl, long long ku) { return (int)((kl + ku + 1 + 31) / 32); }

// u = w[d]; w[d] = w[0]  (the interchange of rows j and j+d, 0 < d <= KL), by
// predicated selects: a switch over d would keep two copies of the window live.
template <typename T, int KL>
__device__ __forceinline__ T reg_interchange(RegArr<T, KL + 1>& w, int d) {
  const T w0 = w[0];
  T u = w0;
#pragma unroll
  for (int p = 1; p <= KL; ++p) {
    const bool h = p == d;
    u = h ? w[p] : u;
    w[p] = h ? w0 : w[p];
  }
  return u;
}

// w[k] = v for a k of the size class KL, by selects over the class's positions (an
// indexed jump costs several hundred cycles).
template <typename T, int KL>
__device__ __forceinline__ void reg_set(RegArr<T, KL + 1>& w, int k, T v) {
  constexpr int lo = reg_cls_lo(KL);
#pragma unroll
  for (int p = lo; p <= KL; ++p) w[p] = p == k ? v : w[p];
}

// The rank-1 update fused with the slide: w[r-1] = fma(l[r-1], nu, w[r]), r = 1..KL.
template <typename T, int KL>
__device__ __forceinline__ void reg_update(RegArr<T, KL + 1>& w, const T* __restrict__ l, T nu) {
  using V = RegVec<T>;
#pragma unroll
  for (int q = 0; q < KL; q += V::n) {
    const typename V::type lv = *reinterpret_cast<const typename V::type*>(l + q);
#pragma unroll
    for (int k = 0; k < V::n; ++k) w[q + k] = fma(V::get(lv, k), nu, w[q + k + 1]);
  }
}

// The same with the plain slide w[r-1] = w[r] where !doit (u == 0 or a zero pivot, as
// dgbtf2 skips those columns), by selects rather than a divergent branch.  The
// multipliers are read from shared memory kRegLookahead vectors ahead of their use,
// so their latency overlaps the arithmetic of the preceding rows.
constexpr int kRegLookahead = 4;
template <typename T, int KL>
__device__ __forceinline__ void reg_update_sel(RegArr<T, KL + 1>& w, const T* __restrict__ l, T nu, bool doit) {
  using V = RegVec<T>;
  using VT = typename V::type;
  constexpr int NG = KL / V::n, D = kRegLookahead < NG ? kRegLookahead : NG;
  const VT* lv = reinterpret_cast<const VT*>(l);
  VT buf[D];
#pragma unroll
  for (int g = 0; g < D; ++g) buf[g] = lv[g];
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    const VT cur = buf[g % D];
    if (g + D < NG) buf[g % D] = lv[g + D];
#pragma unroll
    for (int k = 0; k < V::n; ++k) {
      const int q = g * V::n + k;
      const T f = fma(V::get(cur, k), nu, w[q + 1]);
      w[q] = doit ? f : w[q + 1];
    }
  }
}

// The same with a branch: for the solves, where b(j) == 0 is rare.
template <typename T, int KL>
__device__ __forceinline__ void reg_update_br(RegArr<T, KL + 1>& w, const T* __restrict__ l, T nu, bool doit) {
  using V = RegVec<T>;
  using VT = typename V::type;
  if (doit) {
    constexpr int NG = KL / V::n, D = kRegLookahead < NG ? kRegLookahead : NG;
    const VT* lv = reinterpret_cast<const VT*>(l);
    VT buf[D];
#pragma unroll
    for (int g = 0; g < D; ++g) buf[g] = lv[g];
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      const VT cur = buf[g % D];
      if (g + D < NG) buf[g % D] = lv[g + D];
#pragma unroll
      for (int k = 0; k < V::n; ++k) w[g * V::n + k] = fma(V::get(cur, k), nu, w[g * V::n + k + 1]);
    }
  } else {
#pragma unroll
    for (int r = 1; r <= KL; ++r) w[r - 1] = w[r];
  }
}

template <typename T, int KL>
__device__ __forceinline__ void reg_shift(RegArr<T, KL + 1>& w) {
#pragma unroll
  for (int r = 1; r <= KL; ++r) w[r - 1] = w[r];
}

// Warp argmax, first index on ties (see warp_argmax_first); a Float32 key fits 32 bits,
// so two reductions suffice.
__device__ __forceinline__ int reg_argmax(unsigned long long key, int idx, double) {
  return warp_argmax_first(key, idx);
}
__device__ __forceinline__ int reg_argmax(unsigned long long key, int idx, float) {
  const unsigned k = key > 0xffffffffull ? 0xffffffffu : (unsigned)key;
  const unsigned mk = __reduce_max_sync(0xffffffffu, k);
  return (int)__reduce_min_sync(0xffffffffu, k == mk ? (unsigned)idx : 0x7fffffffu);
}

// Pivot of step jn.  Narrow windows (KL <= 8): the lane holding column jn scans its
// own registers.  Wider: its warp transposes the column through shared memory and
// reduces across lanes.  Either way: idamax over rows 0..km (first index of the
// largest |a|), the interchange inside the column, scaling by the reciprocal of the
// pivot, the step record for the other lanes, and the L column, U(jn,jn) and ipiv in
// memory.
template <typename T, int KL, int NLMAX>
__device__ __forceinline__ void reg_pivot(i64 jn, int ol, int lane, i64 m, int kl, int kv, const RegArr<T, KL + 1>& w,
                                          T* __restrict__ ab, i64 ldab, i64* __restrict__ ipiv,
                                          RegShared<T, KL, NLMAX>& sh) {
  using V = RegVec<T>;
  using VT = typename V::type;
  const int km = (int)min((i64)kl, m - 1 - jn);
  RegStep<T, KL>& rec = sh.rec[jn & 1];
  T* colj = ab + jn * ldab + kv;
  if constexpr (KL <= 8) {
    if (lane != ol) return;
    unsigned long long key = pivot_key(w[0], true);
    int d = 0;
    T piv = w[0];
#pragma unroll
    for (int p = 1; p <= KL; ++p) {
      const unsigned long long k = pivot_key(w[p], false);
      const bool better = p <= km && k > key;
      key = better ? k : key;
      d = better ? p : d;
      piv = better ? w[p] : piv;
    }
    const bool ns = is_nonzero(piv);
    const T rcp = T(1) / (ns ? piv : T(1));
    const T w0 = w[0];
    T l[KL];
#pragma unroll
    for (int p = 1; p <= KL; ++p) {
      const T v = p == d ? w0 : w[p];
      l[p - 1] = ns ? rcp * v : v;
    }
#pragma unroll
    for (int q = 0; q < KL; q += V::n) {
      VT v;
      if constexpr (V::n == 4) v = make_float4(l[q], l[q + 1], l[q + 2], l[q + 3]);
      else v = make_double2(l[q], l[q + 1]);
      *reinterpret_cast<VT*>(rec.l + q) = v;
    }
    rec.d = d;
    rec.ns = ns ? 1 : 0;
#pragma unroll
    for (int p = 1; p <= KL; ++p)
      if (p <= km) colj[p] = l[p - 1];
    colj[0] = piv;
    ipiv[jn] = jn + d + 1;
    if (!ns && sh.info == 0) sh.info = jn + 1;
  } else {
    constexpr int NP = (KL + 1 + 31) / 32;  // rows per lane
    if (lane == ol) {
#pragma unroll
      for (int q = 0; q < KL; q += V::n) {
        VT v;
        if constexpr (V::n == 4) v = make_float4(w[q], w[q + 1], w[q + 2], w[q + 3]);
        else v = make_double2(w[q], w[q + 1]);
        *reinterpret_cast<VT*>(sh.scr + q) = v;
      }
      sh.scr[KL] = w[KL];
    }
    __syncwarp();
    T v[NP];
    unsigned long long key = 0ull;
    int idx = 0x7fffffff;
    T cand = T(1);
#pragma unroll
    for (int k = 0; k < NP; ++k) {
      const int p = lane + 32 * k;
      v[k] = p <= KL ? sh.scr[p] : T(0);
      const unsigned long long kk = pivot_key(v[k], p == 0);
      if (p <= km && (idx == 0x7fffffff || kk > key)) {
        key = kk;
        idx = p;
        cand = v[k];
      }
    }
    // every lane divides by its own candidate while the reduction runs; the winner's
    // quotient is dgbtf2's 1/pivot
    const T crcp = T(1) / (is_nonzero(cand) ? cand : T(1));
    const int d = reg_argmax(key, idx, T(0));
    const T piv = __shfl_sync(0xffffffffu, cand, d & 31);
    const T rcp = __shfl_sync(0xffffffffu, crcp, d & 31);
    const T v0 = __shfl_sync(0xffffffffu, v[0], 0);
    const bool ns = is_nonzero(piv);
#pragma unroll
    for (int k = 0; k < NP; ++k) {
      const int p = lane + 32 * k;
      if (p >= 1 && p <= km) {
        T x = p == d ? v0 : v[k];
        if (ns) x = rcp * x;
        rec.l[p - 1] = x;
        colj[p] = x;
      }
    }
    if (lane == 0) {
      rec.d = d;
      rec.ns = ns ? 1 : 0;
      ipiv[jn] = jn + d + 1;
      colj[0] = piv;
      if (!ns && sh.info == 0) sh.info = jn + 1;
    }
  }
}

// The factorization by one group: tid in [0, NL), NL = 32 * warps >= kl+ku+1; `cta`:
// the group is the whole CTA (else one warp).  Returns dgbtf2's info.
template <typename T, int KL, int NLMAX>
__device__ __noinline__ i64 gbtrf_reg(i64 m, i64 n, int kl, int ku, T* __restrict__ ab, i64 ldab, i64* __restrict__ ipiv,
                         RegShared<T, KL, NLMAX>& sh, int tid, int NL, bool cta) {
  constexpr int P = kRegPre;
  const int kv = kl + ku, lane = tid & 31, wig = tid >> 5;
  const i64 mn = min(m, n);
  if (mn <= 0) return 0;
  auto bar = [&]() {
    if (cta) __syncthreads();
    else __syncwarp();
  };
  // dgbtf2 zeroes the fill rows of columns ku+1 .. mn-1+kv; the U stores below cover the
  // rows < mn, so only rows >= mn (m < n) are cleared here.
  for (i64 c = mn + ku + 1 + tid; c < min(mn + kv, n); c += NL)
    for (i64 i = max(mn, c - kv); i <= c - ku - 1; ++i) ab[(kv + i - c) + c * ldab] = T(0);

  RegArr<T, KL + 1> w;
  {
    const i64 c = tid;
    const bool have = c <= kv && c < n;
#pragma unroll
    for (int r = 0; r <= KL; ++r) {
      T v = T(0);
      if (have && r <= kl && r < m && r >= c - ku) v = ab[(kv + r - c) + c * ldab];
      w[r] = v;
    }
  }
  // E(s): the value entering at the end of step s, row s+1+kl of this lane's column at
  // step s+1 (rel1 = its rel there), zero outside the matrix.  It is loaded P steps
  // ahead into a register, parked in this lane's slot of a shared-memory ring one step
  // later (when the load has landed) and read at step s.
  auto load_e = [&](i64 s, int rel1) -> T {
    const i64 cc = s + 1 + rel1;
    const bool ok = s + 1 < mn && rel1 <= kv && cc < n && s + 1 + kl < m;
    return ok ? ab[(kv + s + 1 + kl - cc) + cc * ldab] : T(0);
  };
  // x mod NL for -NL <= x < NL (an integer division here would cost more than a step)
  auto modnl = [&](int x) { return x < 0 ? x + NL : x; };
  T* ring = sh.pre + tid;
  for (int s = 0; s < P - 1; ++s) ring[s * NL] = load_e(s, modnl(tid - s - 1));
  T nxt = load_e(P - 1, modnl(tid - P));
  if (tid == 0) sh.info = 0;
  if (cta) __syncthreads();
  if (wig == 0) reg_pivot<T, KL, NLMAX>(0, 0, lane, m, kl, kv, w, ab, ldab, ipiv, sh);
  bar();

  int rel = tid;  // (tid - j) mod NL: this lane's column is j + rel
  int o = 0;      // j mod NL: the lane of the pivot column
  for (i64 j = 0; j < mn; ++j) {
    const RegStep<T, KL>& rc = sh.rec[j & 1];
    const int d = rc.d;
    const bool ns = rc.ns != 0;
    const i64 c = j + rel;
    const bool live = rel > 0 && rel <= kv && c < n;
    const int rel1 = rel == 0 ? NL - 1 : rel - 1;
    const bool more = j + 1 < mn;
    ring[(int)((j + P - 1) & (P - 1)) * NL] = nxt;
    nxt = load_e(j + P, modnl(rel - P - 1));
    const T ent = ring[(int)(j & (P - 1)) * NL];
    // interchange, U(j, c), update and slide; lanes without a live column compute
    // values that are never read
    T u = w[0];
    if (ns && d != 0) u = reg_interchange<T, KL>(w, d);
    if (live) ab[(kv + j - c) + c * ldab] = u;
    reg_update_sel<T, KL>(w, rc.l, -u, live && ns && is_nonzero(u));
    if (rel1 == kv) {  // a column enters the window: its rows above the band are zero
#pragma unroll
      for (int r = 0; r <= KL; ++r) w[r] = T(0);
    }
    reg_set<T, KL>(w, kl, ent);
    rel = rel1;
    if (!more) break;
    o = o + 1 == NL ? 0 : o + 1;
    if (wig == (o >> 5)) reg_pivot<T, KL, NLMAX>(j + 1, o & 31, lane, m, kl, kv, w, ab, ldab, ipiv, sh);
    bar();
  }
  if (cta) __syncthreads();
  return sh.info;
}

// ------------------------------------------------------------ solves, trans = 'N'
// One warp; lane r sweeps right-hand side r (nr <= R <= 32) keeping its window of b in
// registers, exactly as the factorization keeps a column: the forward sweep (dgbtrs:
// interchange, then b(j+1:j+lm) -= b(j) * l, skipped when b(j) == 0) with rows j..j+kl,
// the back substitution (dtbsv 'U','N': x(j) /= U(j,j), then x(j-p) -= x(j) * U(j-p,j),
// skipped when x(j) == 0) with rows j..j-kv.  The pivots and L or U columns of a chunk
// of steps and the rows of b entering the window are copied to shared memory with
// cp.async one chunk ahead (two buffers).
template <typename T>
__host__ __device__ constexpr int reg_chunk() { return sizeof(T) == 4 ? 32 : 16; }

template <typename T, int KL, int R = 32>
struct __align__(16) RegFwdStage {
  static constexpr int C = reg_chunk<T>();
  T l[C][KL];       // multipliers of step j0+i, rows 1..KL
  T e[C][R];        // row j0+i+1+kl of b, entering the window, per right-hand side
  long long ip[C];  // ipiv(j0+i)
};
template <typename T, int KV, int R = 32>
struct __align__(16) RegBwdStage {
  static constexpr int C = reg_chunk<T>();
  T u[C][KV];  // U(j-p, j), p = 1..KV, of step j = j0-i
  T e[C][R];   // row j-1-kv of b, entering
  T dg[C];     // U(j, j)
};

template <typename T, int KL, int R>
__device__ __noinline__ void gbtrs_reg_fwd(i64 n, int kl, int ku, int nr, const T* __restrict__ ab, i64 ldab,
                              const i64* __restrict__ ipiv, T* __restrict__ B, i64 ldb,
                              RegFwdStage<T, KL, R> (&st)[2], int lane) {
  constexpr int C = RegFwdStage<T, KL, R>::C;
  if (kl == 0 || n <= 1) return;
  const int kv = kl + ku;
  const bool act = lane < nr;
  T* b = B + (i64)(act ? lane : 0) * ldb;
  auto stage = [&](RegFwdStage<T, KL, R>& S, i64 j0) {
    const int cn = (int)min((i64)C, n - 1 - j0);
    for (int e = lane; e < cn * KL; e += 32) {
      const int i = e / KL, q = e - i * KL;
      const i64 j = j0 + i;
      const bool ok = q < kl && j + 1 + q < n;
      cp_async_elem(&S.l[i][q], ok ? ab + (kv + 1 + q) + j * ldab : ab, ok);
    }
    for (int i = lane; i < cn; i += 32)
      cp_async_elem(&S.ip[i], reinterpret_cast<const long long*>(ipiv) + j0 + i, true);
    for (int e = lane; e < cn * nr; e += 32) {
      const int r = e / cn, i = e - r * cn;
      const i64 row = j0 + i + 1 + kl;
      cp_async_elem(&S.e[i][r], row < n ? B + (i64)r * ldb + row : B, row < n);
    }
    cp_async_commit();
  };
  __syncwarp();
  stage(st[0], 0);
  RegArr<T, KL + 1> w;
#pragma unroll
  for (int r = 0; r <= KL; ++r) w[r] = (act && r <= kl && r < n) ? b[r] : T(0);
  int k = 0;
  for (i64 j0 = 0; j0 < n - 1; j0 += C, k ^= 1) {
    const int cn = (int)min((i64)C, n - 1 - j0);
    cp_async_wait<0>();
    __syncwarp();
    if (j0 + C < n - 1) stage(st[k ^ 1], j0 + C);
    const RegFwdStage<T, KL, R>& S = st[k];
    for (int i = 0; i < cn; ++i) {
      const int d = (int)(S.ip[i] - 1 - (j0 + i));
      T u = w[0];
      if (d != 0) u = reg_interchange<T, KL>(w, d);
      if (act) b[j0 + i] = u;
      reg_update_br<T, KL>(w, S.l[i], -u, is_nonzero(u));
      reg_set<T, KL>(w, kl, S.e[i][lane < R ? lane : 0]);
    }
  }
  if (act) b[n - 1] = w[0];
  __syncwarp();
}

template <typename T, int KV, int R>
__device__ __noinline__ void gbtrs_reg_bwd(i64 n, int kv, int nr, const T* __restrict__ ab, i64 ldab, T* __restrict__ B, i64 ldb,
                              RegBwdStage<T, KV, R> (&st)[2], int lane) {
  constexpr int C = RegBwdStage<T, KV, R>::C;
  if (n <= 0) return;
  const bool act = lane < nr;
  T* b = B + (i64)(act ? lane : 0) * ldb;
  auto stage = [&](RegBwdStage<T, KV, R>& S, i64 j0) {
    const int cn = (int)min((i64)C, j0 + 1);
    for (int e = lane; e < cn * KV; e += 32) {
      const int i = e / KV, q = e - i * KV;
      const bool ok = q < kv;
      cp_async_elem(&S.u[i][q], ok ? ab + (kv - 1 - q) + (j0 - i) * ldab : ab, ok);
    }
    for (int i = lane; i < cn; i += 32) cp_async_elem(&S.dg[i], ab + kv + (j0 - i) * ldab, true);
    for (int e = lane; e < cn * nr; e += 32) {
      const int r = e / cn, i = e - r * cn;
      const i64 row = j0 - i - 1 - kv;
      cp_async_elem(&S.e[i][r], row >= 0 ? B + (i64)r * ldb + row : B, row >= 0);
    }
    cp_async_commit();
  };
  __syncwarp();
  stage(st[0], n - 1);
  RegArr<T, KV + 1> w;  // w[p] = x(j - p)
#pragma unroll
  for (int p = 0; p <= KV; ++p) w[p] = (act && p <= kv && n - 1 - p >= 0) ? b[n - 1 - p] : T(0);
  int k = 0;
  for (i64 j0 = n - 1; j0 >= 0; j0 -= C, k ^= 1) {
    const int cn = (int)min((i64)C, j0 + 1);
    cp_async_wait<0>();
    __syncwarp();
    if (j0 - C >= 0) stage(st[k ^ 1], j0 - C);
    const RegBwdStage<T, KV, R>& S = st[k];
    for (int i = 0; i < cn; ++i) {
      const T x0 = w[0];
      const bool nz = is_nonzero(x0);
      const T xj = nz ? x0 / S.dg[i] : x0;
      if (act) b[j0 - i] = xj;
      reg_update_br<T, KV>(w, S.u[i], -xj, nz);
      reg_set<T, KV>(w, kv, S.e[i][lane < R ? lane : 0]);
    }
  }
  __syncwarp();
}

// ------------------------------------------------------------ per-system dispatch
// For kernels that take systems of different bands: the size class is chosen per
// system.  A group of NL lanes (NL <= NLMAX) factors with the register window when
// kl+ku+1 <= NL; the solve runs in the group's first warp.  `smem` must hold
// reg_smem_bytes<T, NLMAX, R>(kl, ku).
template <typename T>
__host__ __device__ inline bool reg_fits(long long kl, long long ku, int NL) {
  return reg_class<T>(kl, ku) != 0 && kl + ku + 1 <= NL;
}
template <typename T>
__host__ __device__ inline bool reg_solve_fits(long long kl, long long ku) {
  return reg_class<T>(kl, 0) != 0 && reg_kv_class<T>(kl + ku) != 0;
}
template <typename T, int NLMAX, int R>
__host__ __device__ inline long long reg_smem_bytes(long long kl, long long ku) {
  constexpr int KM = reg_kl_max<T>();
  long long f = 0, s = 0, b = 0;
  if (const int kc = reg_class<T>(kl, ku))
    f = reg_dispatch<KM>(kc, [&](auto k) { return (long long)sizeof(RegShared<T, decltype(k)::v, NLMAX>); });
  if (reg_solve_fits<T>(kl, ku)) {
    s = reg_dispatch<KM>(reg_class<T>(kl, 0), [&](auto k) { return 2 * (long long)sizeof(RegFwdStage<T, decltype(k)::v, R>); });
    b = reg_dispatch<2 * KM>(reg_kv_class<T>(kl + ku),
                             [&](auto k) { return 2 * (long long)sizeof(RegBwdStage<T, decltype(k)::v, R>); });
  }
  return f > s ? (f > b ? f : b) : (s > b ? s : b);
}

// Bytes covering every system whose band is within (kl_max, ku_max).
template <typename T, int NLMAX, int R>
inline long long reg_group_bytes(long long kl_max, long long ku_max) {
  long long m = 0;
  const long long km = kl_max < reg_kl_max<T>() ? kl_max : reg_kl_max<T>();
  for (long long kl = 0; kl <= km; ++kl) {
    const long long kum = ku_max < 2 * reg_kl_max<T>() - kl ? ku_max : 2 * reg_kl_max<T>() - kl;
    for (long long ku = 0; ku <= kum; ku += (ku + 16 <= kum ? 16 : 1)) {
      const long long b = reg_smem_bytes<T, NLMAX, R>(kl, ku);
      m = b > m ? b : m;
    }
    const long long b = reg_smem_bytes<T, NLMAX, R>(kl, kum);
    m = b > m ? b : m;
  }
  return m;
}

template <typename T, int NLMAX>
__device__ i64 gbtrf_reg_any(i64 m, i64 n, int kl, int ku, T* ab, i64 ldab, i64* ipiv, void* smem, int tid, int NL,
                             bool cta) {
  return reg_dispatch<reg_kl_max<T>()>(reg_class<T>(kl, ku), [&](auto k) -> i64 {
    constexpr int K = decltype(k)::v;
    return gbtrf_reg<T, K, NLMAX>(m, n, kl, ku, ab, ldab, ipiv, *reinterpret_cast<RegShared<T, K, NLMAX>*>(smem), tid,
                                  NL, cta);
  });
}

// gbtrs 'N' for nr right-hand sides (any number; R at a time) by one warp.
template <typename T, int R>
__device__ void gbtrs_reg_any(i64 n, int kl, int ku, int nr, const T* ab, i64 ldab, const i64* ipiv, T* B, i64 ldb,
                              void* smem, int lane) {
  for (int r0 = 0; r0 < nr; r0 += R) {
    const int q = min(R, nr - r0);
    T* Bq = B + (i64)r0 * ldb;
    reg_dispatch<reg_kl_max<T>()>(reg_class<T>(kl, 0), [&](auto k) {
      constexpr int K = decltype(k)::v;
      gbtrs_reg_fwd<T, K, R>(n, kl, ku, q, ab, ldab, ipiv, Bq, ldb, *reinterpret_cast<RegFwdStage<T, K, R>(*)[2]>(smem),
                             lane);
      return 0;
    });
    reg_dispatch<2 * reg_kl_max<T>()>(reg_kv_class<T>(kl + ku), [&](auto k) {
      constexpr int K = decltype(k)::v;
      gbtrs_reg_bwd<T, K, R>(n, kl + ku, q, ab, ldab, Bq, ldb, *reinterpret_cast<RegBwdStage<T, K, R>(*)[2]>(smem),
                             lane);
      return 0;
    });
  }
}

}  // namespace bm

namespace bm {
// Host launchers (lureg.cu): the factorization of one system by one CTA of
// reg_warps(kl, ku) warps; callers check reg_class<T>(kl, ku) != 0 first.
template <typename T>
int gbtrf_reg_run(i64 m, i64 n, i64 kl, i64 ku, T* ab, i64 ldab, i64* ipiv, i64* info, cudaStream_t stream,
                  const char* name);
// Tiny bands (lureg.cu): kl >= 1 and kl * (kl + ku + 1) <= 32 for the factorization (one
// warp, a lane per window element), kl + ku + 1 <= 32 for the 'N' solve (a warp per
// right-hand side).
__host__ __device__ inline bool tiny_fits(long long kl, long long ku) {
  return kl >= 1 && ku >= 0 && kl * (kl + ku + 1) <= 32;
}
__host__ __device__ inline bool tiny_solve_fits(long long kl, long long ku) {
  return kl >= 0 && ku >= 0 && kl + ku + 1 <= 32;
}
template <typename T>
int gbtrf_tiny_run(i64 m, i64 n, i64 kl, i64 ku, T* ab, i64 ldab, i64* ipiv, i64* info, cudaStream_t stream,
                   const char* name);
template <typename T>
int gbtrs_tiny_run(i64 n, i64 kl, i64 ku, i64 nrhs, const T* ab, i64 ldab, const i64* ipiv, T* B, i64 ldb,
                   cudaStream_t stream, const char* name);
// gbtrs 'N' by one warp per 32 right-hand sides; callers check reg_class<T>(kl, 0) and
// reg_kv_class<T>(kl + ku) first.
template <typename T>
int gbtrs_reg_run(i64 n, i64 kl, i64 ku, i64 nrhs, const T* ab, i64 ldab, const i64* ipiv, T* B, i64 ldb,
                  cudaStream_t stream, const char* name);
}  // namespace bm
