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

// Size classes of the register window and the lanes a band needs.
constexpr int kRegMaxWarps = 8;
template <typename T>
__host__ __device__ constexpr int reg_kl_max() { return sizeof(T) == 4 ? 64 : 32; }
template <typename T>
__host__ __device__ inline int reg_class(long long kl, long long ku) {
  if (kl < 0 || ku < 0 || kl > reg_kl_max<T>() || kl + ku + 1 > 32 * kRegMaxWarps) return 0;
  return kl <= 4 ? 4 : kl <= 8 ? 8 : kl <= 16 ? 16 : kl <= 32 ? 32 : 64;
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

#define BM_RE1(p) \
  case p:                       \
    if constexpr ((p) <= KL) {  \
      w[p] = v;                 \
    }                           \
    break;
#define BM_RE4(p) BM_RE1(p) BM_RE1(p + 1) BM_RE1(p + 2) BM_RE1(p + 3)
#define BM_RE16(p) BM_RE4(p) BM_RE4(p + 4) BM_RE4(p + 8) BM_RE4(p + 12)
#define BM_RE64(p) BM_RE16(p) BM_RE16(p + 16) BM_RE16(p + 32) BM_RE16(p + 48)

// w[k] = v  (k <= KL)
template <typename T, int KL>
__device__ __forceinline__ void reg_set(RegArr<T, KL + 1>& w, int k, T v) {
  switch (k) {
    BM_RE64(0)
    BM_RE64(64)
    BM_RE1(128)
    default:
      break;
  }
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
// dgbtf2 skips those columns), by selects rather than a divergent branch.
template <typename T, int KL>
__device__ __forceinline__ void reg_update_sel(RegArr<T, KL + 1>& w, const T* __restrict__ l, T nu, bool doit) {
  using V = RegVec<T>;
#pragma unroll
  for (int q = 0; q < KL; q += V::n) {
    const typename V::type lv = *reinterpret_cast<const typename V::type*>(l + q);
#pragma unroll
    for (int k = 0; k < V::n; ++k) {
      const T f = fma(V::get(lv, k), nu, w[q + k + 1]);
      w[q + k] = doit ? f : w[q + k + 1];
    }
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
__device__ i64 gbtrf_reg(i64 m, i64 n, int kl, int ku, T* __restrict__ ab, i64 ldab, i64* __restrict__ ipiv,
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

}  // namespace bm

namespace bm {
// Host launchers (lureg.cu): the factorization of one system by one CTA of
// reg_warps(kl, ku) warps; callers check reg_class<T>(kl, ku) != 0 first.
template <typename T>
int gbtrf_reg_run(i64 m, i64 n, i64 kl, i64 ku, T* ab, i64 ldab, i64* ipiv, i64* info, cudaStream_t stream,
                  const char* name);
}  // namespace bm
