// Banded LU (xGBTF2 semantics) and solves (xGBTRS) executed by a group of G warps
// (G = 1: one warp; G > 1: the whole CTA, one warp per SM sub-partition, so a wide
// band gets the SM's full FP64/FP32 throughput).  Shared by the single-system entry
// points, the batched persistent kernels and the mixed-precision solve.
//
// gbtrf: the active part of the matrix at step j is the (kl+1) x (kl+ku+1) window
// A(j:j+kl, j:j+kl+ku); it lives in shared memory as a ring in both dimensions
// (logical row r <-> physical (j+r) mod (kl+1), logical column c <-> (j+c) mod
// (kl+ku+1)), so the window slides one row and one column per step without moving
// data.  The row that enters at each step is fetched P steps ahead with cp.async
// into a staging ring.  Each thread owns whole window columns; a step is two group
// barriers (column 0's multipliers, then every column's interchange, update and slide,
// with the next pivot found by the owner of the next column).  The arithmetic is
// LAPACK's dgbtf2 operation for operation: idamax (first index of the largest |a|), row
// interchange, scaling by the reciprocal of the pivot, and the rank-1 update
// a <- fma(l_i, -u_c, a) skipping u_c == 0 -- so factors and pivots equal the oracle's
// bit for bit.  A panel form (gbtrf_blocked_group; and, across the GPU for bands whose
// window exceeds shared memory, lu.cu's panel + replay kernels) keeps the same
// per-element sequence.
//
// gbtrs: the sweeps are sequential in j and run in chunks of up to kChunk steps: the
// group stages a chunk's L or U columns, pivots and rows of b through shared memory,
// then each warp sweeps its own right-hand sides with warp-level synchronisation (or,
// for few right-hand sides on a wide band, the whole group shares each column's rows).
// Every element receives its updates in the same order as in dgbtrs/dtbsv (the
// transposed triangular solve is done in axpy form, which preserves each element's
// accumulation order).  Only the L^T dot products of the transposed solve use a tree
// reduction when kl > 16.
#pragma once
#include "common.cuh"

namespace bm {

// ------------------------------------------------------------ group helpers
template <int G>
struct Grp {
  static constexpr int NT = 32 * G;
  // G == 1: several independent warps per CTA; G > 1: one group per CTA
  static __device__ __forceinline__ int tid() { return G == 1 ? (int)(threadIdx.x & 31) : (int)threadIdx.x; }
  static __device__ __forceinline__ void sync() {
    if (G == 1) __syncwarp();
    else __syncthreads();
  }
};

// Next work item for the calling group (an atomic counter), broadcast to the group
// through hdr (the group's shared-memory header).
template <int G>
__device__ __forceinline__ int next_item(int32_t* counter, int* hdr) {
  int idx = 0;
  if (Grp<G>::tid() == 0) idx = atomicAdd(counter, 1);
  if (G == 1) return __shfl_sync(0xffffffffu, idx, 0);
  if (threadIdx.x == 0) hdr[1] = idx;
  __syncthreads();
  idx = hdr[1];
  __syncthreads();
  return idx;
}

// Legality of one batch descriptor for a group whose shared memory was sized for
// bandwidths up to (bound_kl, bound_ku): 0, or -(field number) of the first illegal
// field (n 1, kl 2, ku 3, nrhs 4, ab_offset 5, ldab 6, b_offset 7, ldb 8,
// ipiv_offset 9), which the batched kernels store as the system's info and skip the
// system.  A band wider than the bound would run past the group's shared memory.
__device__ __forceinline__ i64 desc_check(const bm_gb_desc& d, i64 bound_kl, i64 bound_ku) {
  if (d.n < 0 || d.n > 0x7fffffffLL) return -1;
  if (d.kl < 0 || d.kl > bound_kl) return -2;
  if (d.ku < 0 || d.ku > bound_ku) return -3;
  if (d.nrhs < 0 || d.nrhs > 0x7fffffffLL) return -4;
  if (d.ab_offset < 0) return -5;
  if (d.ldab < 2 * d.kl + d.ku + 1) return -6;
  if (d.b_offset < 0) return -7;
  if (d.ldb < (d.n > 1 ? d.n : 1)) return -8;
  if (d.ipiv_offset < 0) return -9;
  return 0;
}

// Group-wide maximum (NaN propagates); scratch: G doubles of shared memory.
template <int G>
__device__ __forceinline__ double grp_max(double v, double* scratch) {
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    const double o = __shfl_xor_sync(0xffffffffu, v, off);
    v = (o > v || o != o) ? o : v;
  }
  if (G == 1) return v;
  const int w = threadIdx.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) scratch[w] = v;
  __syncthreads();
  v = scratch[0];
  for (int k = 1; k < G; ++k) v = (scratch[k] > v || scratch[k] != scratch[k]) ? scratch[k] : v;
  __syncthreads();
  return v;
}

// |a| as an integer key whose order is the order of |a| (IEEE bit pattern, sign cleared).
__device__ __forceinline__ unsigned long long abs_key(double a) {
  return (unsigned long long)__double_as_longlong(a) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ unsigned long long abs_key(float a) {
  return (unsigned long long)(__float_as_uint(a) & 0x7fffffffu);
}
// The key idamax's scan compares: |a| by bit pattern, except that a NaN never wins
// (both |x| > NaN and NaN > |x| are false in the scan) unless it is the first entry,
// which the scan starts from and nothing then exceeds.
__device__ __forceinline__ unsigned long long pivot_key(double a, bool first) {
  const unsigned long long k = abs_key(a);
  return k > 0x7ff0000000000000ull ? (first ? ~0ull : 0ull) : k;
}
__device__ __forceinline__ unsigned long long pivot_key(float a, bool first) {
  const unsigned long long k = abs_key(a);
  return k > 0x7f800000ull ? (first ? ~0ull : 0ull) : k;
}
// a != 0 (either sign of zero) without a floating-point compare
__device__ __forceinline__ bool is_nonzero(double a) { return (abs_key(a)) != 0ull; }
__device__ __forceinline__ bool is_nonzero(float a) { return (abs_key(a)) != 0ull; }

// ---- division by a staged reciprocal (Float64)
// On GB300's FP64 pipe a division costs about 570 cycles of latency and an fma 64.
// Where the divisor d is known ahead of the step that divides by it (U(j,j) in a
// solve), its reciprocal pair is staged off the critical path:
//   yh = RN(1/d),  e = 1 - d*yh (exact, by fma),  yl = RN(e*yh),
// and x/d, correctly rounded, then takes four dependent operations:
//   t = RN(x*yl);  q0 = RN(x*yh + t);  r = x - d*q0 (exact);  q = RN(q0 + r*yh).
// With Q = x/d in binade 2^eq and md the significand of d:
//   * yh + yl is within 2^-105 |1/d| of 1/d, so q0 is within half an ulp of Q plus
//     2^-50.4 of that, and r is exactly representable (a multiple of ulp(d) ulp(q0)
//     below 2^53 of them);
//   * q = RN(Q + r (yh - 1/d)), an error below md 2^(eq-107) (1 + 2^-50.4);
//   * Q is at least 2^(eq-105)/md away from every midpoint between doubles (x - d*mid
//     is a nonzero multiple of 2^(ed+eq-105), as mid has 54 significant bits);
// so q = RN(Q) whenever md <= 2 - 2^-48 (Markstein's correction step; Muller et al.,
// Handbook of Floating-Point Arithmetic, ch. 4).  That holds for every d but the 15
// largest significands; those, subnormal or non-finite operands and exponents beyond
// +-900 (where a step could underflow) take the plain x / d.
__device__ __forceinline__ void div_rcp(double d, double& yh, double& yl) {
  yh = 1.0 / d;
  yl = fma(-d, yh, 1.0) * yh;
}
__device__ __forceinline__ double div_staged(double x, double d, double yh, double yl) {
  const unsigned long long bx = (unsigned long long)__double_as_longlong(x);
  const unsigned long long bd = (unsigned long long)__double_as_longlong(d);
  const int ex = (int)((bx >> 52) & 0x7ff) - 1023, ed = (int)((bd >> 52) & 0x7ff) - 1023;
  const bool ok = ex >= -900 && ex <= 900 && ed >= -900 && ed <= 900 && ex - ed >= -900 && ex - ed <= 900 &&
                  (bd & 0xfffffffffffffull) <= 0xffffffffffff0ull;
  if (!ok) return x / d;
  const double q0 = fma(x, yh, x * yl);
  const double r = fma(-d, q0, x);
  return fma(r, yh, q0);
}
__device__ __forceinline__ void div_rcp(float d, float& yh, float& yl) {
  yh = d;
  yl = 0.0f;
}
__device__ __forceinline__ float div_staged(float x, float d, float, float) { return x / d; }

// Warp argmax with the first index winning ties (idamax): every lane passes its best
// (key, index); lanes with nothing to offer pass index 0x7fffffff.  Returns the winning
// index to all lanes, using redux.sync on the integer pipe.
__device__ __forceinline__ int warp_argmax_first(unsigned long long key, int idx) {
  const unsigned hi = (unsigned)(key >> 32), lo = (unsigned)key;
  const unsigned mhi = __reduce_max_sync(0xffffffffu, hi);
  const unsigned mlo = __reduce_max_sync(0xffffffffu, hi == mhi ? lo : 0u);
  const bool cand = (hi == mhi) && (lo == mlo);
  return (int)__reduce_min_sync(0xffffffffu, cand ? (unsigned)idx : 0x7fffffffu);
}

// Shared-memory footprints, in elements of T.  Every group region starts with a
// kHdr-element header (scalars broadcast between the group's warps).
constexpr int kHdr = 16;
__host__ __device__ inline int lu_rs(int kl) { return (kl + 1) | 1; }  // odd column stride: no bank conflicts
template <int P>
__host__ __device__ inline i64 gbtrf_smem_elems(int kl, int ku) {
  const int K = kl + ku + 1;
  // header + window + staging ring + the step's multipliers (kl+1)
  return kHdr + (i64)lu_rs(kl) * K + (i64)P * K + (kl + 1);
}

constexpr int kChunk = 32;  // solve steps staged per chunk (at most)
constexpr int kMaxRhs = 8;  // right-hand sides swept together
__host__ __device__ inline i64 gbtrs_smem_elems(int kl, int ku, int ch = kChunk) {
  const int kv = kl + ku;
  // header + ipiv chunk (kChunk int64, as 2*kChunk T slots) + window of b
  // ((ch+kv+1) rows x kMaxRhs) + chunk of L or U columns (ch x (kv+1))
  return kHdr + 2 * kChunk + (i64)(ch + kv + 1) * kMaxRhs + (i64)ch * (kv + 1);
}
// the largest chunk (<= kChunk) whose solve window fits `bytes` of shared memory, 0 if none
template <typename T>
inline int gbtrs_chunk_for(int kl, int ku, i64 bytes) {
  for (int ch = kChunk; ch >= 1; ch >>= 1)
    if (gbtrs_smem_elems(kl, ku, ch) * (i64)sizeof(T) <= bytes) return ch;
  return 0;
}

// X[s] <- X[s + d] for s in [0, count), d >= 0 (group-cooperative, overlap-safe)
template <typename T, int G>
__device__ __forceinline__ void grp_shift_down(T* X, int count, int d) {
  const int t = Grp<G>::tid();
  for (int s0 = 0; s0 < count; s0 += Grp<G>::NT) {
    const int s = s0 + t;
    const T v = (s < count) ? X[s + d] : T(0);
    Grp<G>::sync();
    if (s < count) X[s] = v;
    Grp<G>::sync();
  }
}
// X[s + d] <- X[s] for s in [0, count), d >= 0, processed from the top
template <typename T, int G>
__device__ __forceinline__ void grp_shift_up(T* X, int count, int d) {
  const int t = Grp<G>::tid();
  for (int s0 = count - 1; s0 >= 0; s0 -= Grp<G>::NT) {
    const int s = s0 - t;
    const T v = (s >= 0) ? X[s] : T(0);
    Grp<G>::sync();
    if (s >= 0) X[s + d] = v;
    Grp<G>::sync();
  }
}

// a[r] = fma(l[r], nu, a[r]) for r < len; chunks of 8 with every load of a chunk
// issued before its stores (a and l never overlap)
template <typename T>
__device__ __forceinline__ void rank1_run(T* a, const T* l, int len, T nu) {
  constexpr int kU = 8;
  int r = 0;
  for (; r + kU <= len; r += kU) {
    T lv[kU], av[kU];
#pragma unroll
    for (int q = 0; q < kU; ++q) {
      lv[q] = l[r + q];
      av[q] = a[r + q];
    }
#pragma unroll
    for (int q = 0; q < kU; ++q) a[r + q] = fma(lv[q], nu, av[q]);
  }
  for (; r < len; ++r) a[r] = fma(l[r], nu, a[r]);
}

// --------------------------------------------------------------------- gbtrf
// Factors the m x n band in ab (LAPACK gbtrf storage, ldab >= 2kl+ku+1) in place;
// writes 1-based pivots to ipiv[0..min(m,n)) and returns LAPACK's info (to every
// thread of the group).
//
// Step j works on the window W (logical rows 0..kl = matrix rows j..j+kl, logical
// columns 0..kv = matrix columns j..j+kv).  Physical window column p is owned by
// thread p mod NT for the whole factorization; a step is two group barriers:
//   phase 1 (all threads, column 0 only): with the pivot row jp known, the multipliers
//     l_r = (1/piv) * a_r (the swapped-in a_jp = old a_0) are written over column 0
//     and stored as L(j+r, j); U(j,j) = piv and ipiv[j] are stored.  The column that
//     left the window last step is cleared for its new role as column kv.
//   phase 2 (each owner, its columns c = 1..kv): swap rows 0 and jp, store U(j, j+c),
//     the update a_r = fma(l_r, -u_c, a_r) (skipped for u_c == 0), and the slide (the
//     entering row's value into the slot row 0 leaves).  The owner of column 1 then
//     finds the next pivot (idamax of the new column 0), so the search is off the
//     critical path of the other columns.
// Columns beyond LAPACK's ju hold u_c = 0 in both swapped rows (nothing has filled
// them), so treating every column like dgbtf2 treats columns <= ju changes no bit.
template <typename T, int P, int G>
__device__ i64 gbtrf_group(i64 m, i64 n, int kl, int ku, T* __restrict__ ab, i64 ldab, i64* __restrict__ ipiv,
                           T* __restrict__ smem) {
  constexpr int NT = Grp<G>::NT;
  const int tid = Grp<G>::tid(), lane = threadIdx.x & 31, wig = tid >> 5;
  const int kv = kl + ku, R = kl + 1, K = kv + 1, RS = lu_rs(kl);
  int* hdr = reinterpret_cast<int*>(smem);
  T* W = smem + kHdr;
  T* S = W + (i64)RS * K;
  T* Lm = S + (i64)P * K;  // multipliers of the step, by logical row (1..km)
  const i64 mn = min(m, n);
  i64 info = 0;
  if (mn <= 0) return 0;

  // initial window: matrix rows 0..kl, columns 0..kv
  for (int e = tid; e < R * K; e += NT) {
    const int c = e / R, r = e - c * R;
    T v = T(0);
    if (r < m && c < n && r - c <= kl && c - r <= ku) v = ab[(kv + r - c) + (i64)c * ldab];
    W[r + c * RS] = v;
  }
  // rows kl+1 .. kl+P into the staging ring (one cp.async group per row and thread)
  auto issue_row = [&](i64 i) {
    T* dst = S + (int)(i & (P - 1)) * K;
    for (int c = tid; c < K; c += NT) {
      const i64 col = i - kl + c;
      const bool ok = i < m && col < n;
      cp_async_elem(dst + c, ok ? ab + (kv + kl - c) + col * ldab : ab, ok);
    }
    cp_async_commit();
  };
  for (int p = 0; p < P; ++p) issue_row((i64)kl + 1 + p);
  Grp<G>::sync();

  // idamax over logical rows 0..km of physical column pc (logical row r at physical
  // (rb + r) mod R), run by the warp that owns pc; the result is returned to that
  // warp's lanes.  Narrow bands: one thread scans with the reference's compares;
  // wider: lanes compare IEEE bit patterns and combine with redux.sync.
  auto find_pivot = [&](int pc, int rb, int km) -> int {
    const T* col = W + pc * RS;
    int jp = 0;
    if (kl <= 8) {
      if (tid == pc % NT) {
        T amax = fabs(col[rb]);
        for (int r = 1; r <= km; ++r) {
          int pr = rb + r;
          pr = pr >= R ? pr - R : pr;
          const T a = fabs(col[pr]);
          if (a > amax) {
            amax = a;
            jp = r;
          }
        }
      }
      jp = __shfl_sync(0xffffffffu, jp, (pc % NT) & 31);
    } else {
      __syncwarp();
      unsigned long long key = 0ull;
      int idx = 0x7fffffff;
      for (int r = lane; r <= km; r += 32) {
        int pr = rb + r;
        pr = pr >= R ? pr - R : pr;
        const unsigned long long k = pivot_key(col[pr], r == 0);
        if (idx == 0x7fffffff || k > key) {
          key = k;
          idx = r;
        }
      }
      jp = warp_argmax_first(key, idx);
    }
    return jp;
  };

  int pr0 = 0, pc0 = 0;
  int jp = 0;
  {
    const int km0 = (int)min((i64)kl, m - 1);
    if (wig == (0 % NT) >> 5) jp = find_pivot(0, 0, km0);
    if (G > 1) {
      if (tid == 0) hdr[0] = jp;
      Grp<G>::sync();
      jp = hdr[0];
    }
  }
  for (i64 j = 0; j < mn; ++j) {
    const int km = (int)min((i64)kl, m - 1 - j);
    const bool last = (j + 1 == mn);
    int prp = pr0 + jp;
    prp = prp >= R ? prp - R : prp;
    T* col0 = W + pc0 * RS;
    const T piv = col0[prp];
    const bool nonsingular = is_nonzero(piv);
    // ---- phase 1: column 0 (multipliers into Lm, L and U(j,j) stores; column 0 itself
    // is only read), and clear the column that left the window at the previous step
    // (physical pc0-1, now logical column kv)
    if (tid == 0) {
      ipiv[j] = j + jp + 1;
      ab[kv + j * ldab] = piv;
    }
    if (km > 0) {
      const T old0 = col0[pr0];
      const T rcp = nonsingular ? T(1) / piv : T(0);
      for (int r = 1 + tid; r <= km; r += NT) {
        int pr = pr0 + r;
        pr = pr >= R ? pr - R : pr;
        T v = (nonsingular && r == jp) ? old0 : col0[pr];
        if (nonsingular) v = rcp * v;
        Lm[r] = v;
        ab[(kv + r) + j * ldab] = v;
      }
    }
    if (!nonsingular && info == 0) info = j + 1;
    if (j > 0) {
      int pcl = pc0 - 1;
      pcl = pcl < 0 ? pcl + K : pcl;
      const int prl = pr0 == 0 ? R - 1 : pr0 - 1;  // holds the row that entered last step
      for (int r = tid; r < R; r += NT)
        if (r != prl) W[r + pcl * RS] = T(0);
    }
    if (!last) cp_async_wait<P - 1>();
    Grp<G>::sync();
    // ---- phase 2: every other column, by its owner
    const i64 inew = j + 1 + kl;
    const T* st = S + (int)(inew & (P - 1)) * K;
    const int ncw = (int)min((i64)kv, n - 1 - j);
    int p1 = pc0 + 1;
    p1 = p1 >= K ? p1 - K : p1;
    for (int pcc = tid; pcc < K; pcc += NT) {
      if (pcc == pc0) {
        if (!last) col0[pr0] = st[kv];  // the new column kv's entry in the entering row
        continue;
      }
      const int c = pcc >= pc0 ? pcc - pc0 : pcc - pc0 + K;
      T* colc = W + pcc * RS;
      T uc = colc[pr0];
      if (nonsingular && jp != 0) {
        const T t = colc[prp];
        colc[prp] = uc;
        uc = t;
      }
      if (c <= ncw) ab[(kv - c) + (j + c) * ldab] = uc;
      if (nonsingular && km > 0 && is_nonzero(uc)) {
        // logical rows 1..km are physical rows pr0+1.. (first segment) and then 0..
        // (after the wrap): two runs with unit stride in both colc and Lm
        const int s1 = min(km, R - 1 - pr0);
        rank1_run<T>(colc + pr0 + 1, Lm + 1, s1, -uc);
        rank1_run<T>(colc, Lm + 1 + s1, km - s1, -uc);
      }
      if (!last) colc[pr0] = st[c - 1];  // slide: the entering row takes row 0's slot
    }
    if (last) break;
    // ---- next pivot, by the warp owning the next column 0 (physical p1)
    {
      const int pr1 = pr0 + 1 == R ? 0 : pr0 + 1;
      const int km1 = (int)min((i64)kl, m - 2 - j);
      int jn = 0;
      if (wig == (p1 % NT) >> 5) jn = find_pivot(p1, pr1, km1);
      if (G > 1) {
        if (tid == p1 % NT) hdr[0] = jn;
      } else {
        jp = jn;
      }
    }
    Grp<G>::sync();
    if (G > 1) jp = hdr[0];
    issue_row(inew + P);
    pr0 = pr0 + 1 == R ? 0 : pr0 + 1;
    pc0 = p1;
  }
  cp_async_wait<0>();
  Grp<G>::sync();
  return info;
}

// ------------------------------------------------------------ blocked gbtrf
// The same factorization in panels of NB columns, for one group of G > 1 warps.
// dgbtf2 gives every element of a column the same sequence per elimination step k:
// the interchange of rows k and k+jp_k, then (for a nonzero pivot and u_k != 0)
// a <- fma(l, -u_k, a) on the rows k+1 .. k+km_k.  The blocked order keeps each
// column's sequence and only regroups columns:
//   * the panel's NB columns take their steps one by one (the interchange of step c
//     over columns c..NB-1 of the panel, the scaling of column c, the rank-1 update of
//     the later panel columns), as dgbtf2 does;
//   * every trailing column then replays the panel's steps k = 0..NB-1 in order --
//     interchange, then its update from the stored multipliers of step k -- one thread
//     per column, all columns at once;
// so factors and pivots equal dgbtf2's bit for bit while the steps that cannot be
// parallelised touch only NB columns.  L columns are stored as each step leaves them
// (dgbtf2's format); U rows when the panel is done.
//
// The window holds rows j0 .. j0+R-1, R = kl+NB, and columns j0 .. j0+C-1, C = kl+ku+NB,
// of the partially factored matrix, as a ring in both dimensions (row r at physical
// (rb + r) mod R, column c at (cb + c) mod C, column stride RS = R|1).
constexpr int kNB = 16;
template <typename T>
__host__ __device__ inline i64 gbtrf_blocked_smem_elems(int kl, int ku) {
  const int R = kl + kNB, C = kl + ku + kNB;
  return kHdr + (i64)(R | 1) * C + 2 * kNB;  // header + window + the panel's pivots and flags
}

template <typename T, int G>
__device__ i64 gbtrf_blocked_group(i64 m, i64 n, int kl, int ku, T* __restrict__ ab, i64 ldab,
                                   i64* __restrict__ ipiv, T* __restrict__ smem) {
  static_assert(G > 1, "blocked gbtrf runs on a whole CTA");
  constexpr int NT = Grp<G>::NT, NB = kNB;
  const int tid = threadIdx.x, lane = tid & 31, wig = tid >> 5;
  const int kv = kl + ku, R = kl + NB, C = kv + NB, RS = R | 1;
  int* hdr = reinterpret_cast<int*>(smem);
  T* W = smem + kHdr;
  int* JP = reinterpret_cast<int*>(W + (i64)RS * C);  // per panel step: pivot offset,
  int* NS = JP + kNB;                                  // and whether the pivot is nonzero
  const i64 mn = min(m, n);
  i64 info = 0;
  if (mn <= 0) return 0;
  int rb = 0, cb = 0;
  auto prow = [&](int r) { int q = rb + r; return q >= R ? q - R : q; };
  auto pcol = [&](int c) { int q = cb + c; return q >= C ? q - C : q; };
  // A(i, c) of the original band (zero outside it); i, c are matrix indices
  auto orig = [&](i64 i, i64 c) -> T {
    return (i < m && c < n && i - c <= kl && c - i <= ku) ? ab[(kv + i - c) + c * ldab] : T(0);
  };
  // initial window: matrix rows 0..R-1, columns 0..C-1
  for (int e = tid; e < R * C; e += NT) {
    const int c = e / R, r = e - c * R;
    W[r + c * RS] = orig(r, c);
  }
  __syncthreads();

  for (i64 j0 = 0; j0 < mn; j0 += NB) {
    const int jb = (int)min((i64)NB, mn - j0);
    // ---- panel: steps c = 0..jb-1 on columns [0, jb) (interchanges over all columns)
    for (int c = 0; c < jb; ++c) {
      const i64 gj = j0 + c;
      const int km = (int)min((i64)kl, m - 1 - gj);
      T* colc = W + pcol(c) * RS;
      if (wig == 0) {  // idamax over rows c..c+km
        unsigned long long key = 0ull;
        int idx = 0x7fffffff;
        for (int r = lane; r <= km; r += 32) {
          const unsigned long long k = pivot_key(colc[prow(c + r)], r == 0);
          if (idx == 0x7fffffff || k > key) {
            key = k;
            idx = r;
          }
        }
        const int jp = warp_argmax_first(key, idx);
        if (lane == 0) {
          hdr[0] = jp;
          JP[c] = jp;
          NS[c] = is_nonzero(colc[prow(c + jp)]) ? 1 : 0;
          ipiv[gj] = gj + jp + 1;
        }
      }
      __syncthreads();
      const int jp = hdr[0];
      const int pr0 = prow(c), prp = prow(c + jp);
      const T piv = colc[prp];
      const bool nonsingular = is_nonzero(piv);
      if (nonsingular && jp != 0)  // interchange rows c and c+jp in panel columns c..jb-1
        for (int t = c + tid; t < jb; t += NT) {
          T* col = W + pcol(t) * RS;
          const T a = col[pr0];
          col[pr0] = col[prp];
          col[prp] = a;
        }
      __syncthreads();
      if (nonsingular) {
        const T rcp = T(1) / piv;
        for (int r = 1 + tid; r <= km; r += NT) colc[prow(c + r)] = rcp * colc[prow(c + r)];
      } else if (info == 0) {
        info = gj + 1;
      }
      __syncthreads();
      for (int r = 1 + tid; r <= km; r += NT) ab[(kv + r) + gj * ldab] = colc[prow(c + r)];  // L(gj+r, gj)
      // rank-1 update of the panel's later columns: thread per (row, column) pair
      if (nonsingular) {
        const int nc = jb - 1 - c;
        for (int e = tid; e < km * nc; e += NT) {
          const int cc = c + 1 + e / km, r = c + 1 + e % km;
          T* col = W + pcol(cc) * RS;
          const T u = col[pr0];
          if (is_nonzero(u)) col[prow(r)] = fma(colc[prow(r)], -u, col[prow(r)]);
        }
      }
      __syncthreads();
    }
    // ---- trailing columns [jb, C): each replays the panel's steps in order
    for (int t = jb + tid; t < C; t += NT) {
      T* col = W + pcol(t) * RS;
      for (int k = 0; k < jb; ++k) {
        if (!NS[k]) continue;  // a zero pivot: no interchange, no update
        const int pk = prow(k);
        T u = col[pk];
        if (JP[k] != 0) {
          const int pp = prow(k + JP[k]);
          const T v = col[pp];
          col[pp] = u;
          u = v;
          col[pk] = u;
        }
        if (!is_nonzero(u)) continue;
        const T nu = -u;
        const T* lk = W + pcol(k) * RS;
        const int len = (int)min((i64)kl, m - 1 - (j0 + k));  // rows k+1 .. k+km_k
        const int p1 = prow(k + 1 >= R ? k + 1 - R : k + 1);  // physical row of k+1
        const int s1 = min(len, R - p1);                        // rows before the wrap
        rank1_run<T>(col + p1, lk + p1, s1, nu);
        rank1_run<T>(col, lk, len - s1, nu);
      }
    }
    __syncthreads();
    // ---- U rows j0 .. j0+jb-1 to global; U(gj, gj+c') = window (r, r + c'), c' <= kv
    for (int e = tid; e < jb * (kv + 1); e += NT) {
      const int r = e / (kv + 1), d = e - r * (kv + 1);
      const i64 gi = j0 + r, gc = gi + d;
      if (gc < n) ab[(kv - d) + gc * ldab] = W[pcol(r + d) * RS + prow(r)];
    }
    if (j0 + jb >= mn) break;
    __syncthreads();
    // ---- slide by NB: rows j0+R.. and columns j0+C.. enter (original band, zero
    // elsewhere) into the slots rows/columns 0..NB-1 leave
    const i64 nj = j0 + NB;
    for (int e = tid; e < NB * C; e += NT) {  // new rows, every new-frame column
      const int rr = e / C, c = e - rr * C;   // new-frame row R-NB+rr, column c
      const int pr = prow(rr), pc = pcol(NB + c >= C ? NB + c - C : NB + c);
      W[pc * RS + pr] = orig(nj + R - NB + rr, nj + c);
    }
    for (int e = tid; e < NB * (R - NB); e += NT) {  // new columns, old rows that stay
      const int cc = e / (R - NB), r = e - cc * (R - NB);  // new-frame column C-NB+cc, row r
      const int pc = pcol(cc), pr = prow(NB + r);
      W[pc * RS + pr] = orig(nj + r, nj + C - NB + cc);
    }
    __syncthreads();
    rb = prow(NB);
    cb = pcol(NB);
  }
  __syncthreads();
  return info;
}

// --------------------------------------------------------------------- gbtrs
// Thread layout for a group of nr <= kMaxRhs right-hand sides: nr is padded to a
// power of two 1 << lg; thread -> (row offset tid >> lg, column tid & ((1<<lg)-1)),
// rows advancing by NT >> lg.  Window element (row s, column c) lives at X[s*nr + c].
__device__ __forceinline__ int rhs_lg(int nr) { return nr <= 1 ? 0 : nr <= 2 ? 1 : nr <= 4 ? 2 : 3; }

// Solves op(A) X = B for nr <= kMaxRhs right-hand sides (B: n x nr, leading dim ldb)
// with the gbtrf factors; trans: false = 'N', true = 'T'.
//
// The sweeps run in chunks of kChunk steps.  At a chunk boundary the whole group
// stages the chunk's L or U columns (LC), its pivots (IP) and the rows of b the chunk
// needs (window X, row-major over the nr columns); inside a chunk each warp sweeps its
// own right-hand-side columns (warp w: columns [w*q, (w+1)*q), q = ceil(nr/G)) with
// only warp-level synchronisation.  Every element receives its updates in dgbtrs /
// dtbsv order.
template <typename T, int G>
__device__ void gbtrs_group(bool trans, i64 n, int kl, int ku, int nr, const T* __restrict__ ab, i64 ldab,
                            const i64* __restrict__ ipiv, T* __restrict__ b, i64 ldb, T* __restrict__ smem,
                            int ch = kChunk) {
  constexpr int NT = Grp<G>::NT;
  const int tid = Grp<G>::tid(), lane = threadIdx.x & 31, wig = tid >> 5;
  const int kv = kl + ku;
  // Column sets: each warp sweeps its own right-hand sides (warp w: columns
  // [w*q, (w+1)*q)) with warp-level synchronisation -- or, when there are far fewer
  // right-hand sides than warps and the band is wide, the whole group shares every
  // column's rows and synchronises as a group ("row split").
  const bool split = G > 1 && nr * 4 <= G && kv >= 192;
  const int SW = split ? NT : 32;           // threads sharing a column set
  const int sl = split ? tid : lane;        // this thread's index in its set
  const int q = split ? nr : (nr + G - 1) / G;
  const int cw0 = split ? 0 : min(nr, wig * q), nw = min(nr, cw0 + q) - cw0;
  // thread -> (column cw0 + (sl & (2^lg-1)), first row sl >> lg), rows advancing by SW >> lg
  const int lg = rhs_lg(nw), cl = cw0 + (sl & ((1 << lg) - 1)), rstep = SW >> lg, r0 = sl >> lg;
  const bool cok = nw > 0 && (sl & ((1 << lg) - 1)) < nw;
  const bool own = sl < nw;  // threads that own one whole column (cw0 + sl)
  const int oc = cw0 + sl;
  auto wsync = [split] {
    if (split) Grp<G>::sync();
    else __syncwarp();
  };
  const int kCh = ch;                             // this call's chunk
  i64* IP = reinterpret_cast<i64*>(smem + kHdr);  // chunk pivots (8-byte aligned)
  T* X = smem + kHdr + 2 * kChunk;                // window: XW rows x nr
  const int XW = kCh + kv + 1;
  T* LC = X + XW * kMaxRhs;                       // chunk columns x (kv+1)
  auto gsync = [] { Grp<G>::sync(); };
  // group-cooperative copies of window rows [s0, s1) from/to b rows g0 + s0 .. (zero
  // outside [0, n))
  auto load_rows = [&](int s0, int s1, i64 g0) {
    const int cnt = (s1 - s0) * nr;
    for (int e = tid; e < cnt; e += NT) {
      const int sr = s0 + e / nr, c = e - (e / nr) * nr;
      const i64 g = g0 + sr;
      X[sr * nr + c] = (g >= 0 && g < n) ? b[g + c * ldb] : T(0);
    }
  };
  auto store_rows = [&](int s0, int s1, i64 g0) {
    const int cnt = (s1 - s0) * nr;
    for (int e = tid; e < cnt; e += NT) {
      const int sr = s0 + e / nr, c = e - (e / nr) * nr;
      const i64 g = g0 + sr;
      if (g >= 0 && g < n) b[g + c * ldb] = X[sr * nr + c];
    }
  };

  if (!trans) {
    // ---- forward: L with row interchanges (dgbtrs 'N': dswap + dger per column)
    if (kl > 0 && n > 1) {
      load_rows(0, kl, 0);
      for (i64 j0 = 0; j0 < n - 1; j0 += kCh) {
        const int jn = (int)min((i64)kCh, n - 1 - j0);
        load_rows(kl, jn + kl, j0);
        for (int sidx = 0; sidx < jn; ++sidx)
          for (int i = tid; i < kl; i += NT)
            cp_async_elem(LC + sidx * kl + i, ab + (kv + 1 + i) + (j0 + sidx) * ldab, j0 + sidx + 1 + i < n);
        cp_async_commit();
        for (int sidx = tid; sidx < jn; sidx += NT) IP[sidx] = ipiv[j0 + sidx] - 1 - j0;
        cp_async_wait<0>();
        gsync();
        if (nw > 0) {
          for (int st = 0; st < jn; ++st) {
            const int lm = (int)min((i64)kl, n - 1 - (j0 + st));
            const int l = (int)IP[st];
            if (l != st) {
              if (own) {
                const T t = X[l * nr + oc];
                X[l * nr + oc] = X[st * nr + oc];
                X[st * nr + oc] = t;
              }
              wsync();
            }
            if (cok) {
              const T bj = X[st * nr + cl];
              if (is_nonzero(bj)) {
                const T t = -bj;
                for (int i = r0; i < lm; i += rstep)
                  X[(st + 1 + i) * nr + cl] = fma(LC[st * kl + i], t, X[(st + 1 + i) * nr + cl]);
              }
            }
            wsync();
          }
        }
        gsync();
        store_rows(0, jn, j0);
        gsync();
        grp_shift_down<T, G>(X, kl * nr, jn * nr);  // carry rows jn .. jn+kl to the front
        if (j0 + jn >= n - 1) store_rows(0, kl, j0 + jn);
        gsync();
      }
    }
    // ---- backward: U x = y (dtbsv 'U','N','N', bandwidth kv), columns n-1 .. 0;
    // window row s <-> b row base + s, with row XW-1 = j1 at the start of each chunk
    i64 j1 = n - 1;
    i64 base = j1 - (XW - 1);
    load_rows(0, XW, base);
    gsync();
    while (true) {
      const int jn = (int)min((i64)kCh, j1 + 1);
      // U(j-i, j) = ab[(kv-i) + j*ldab], i = 0..kv, for j = j1, j1-1, ...
      for (int t = 0; t < jn; ++t) {
        const i64 j = j1 - t;
        for (int i = tid; i <= kv; i += NT) cp_async_elem(LC + t * (kv + 1) + i, ab + (kv - i) + j * ldab, j - i >= 0);
      }
      cp_async_commit();
      // the reciprocal pairs of the chunk's U(j, j), in the pivot slots (unused here)
      T* RH = reinterpret_cast<T*>(IP);
      for (int t = tid; t < jn; t += NT) div_rcp(ab[kv + (j1 - t) * ldab], RH[t], RH[kChunk + t]);
      cp_async_wait<0>();
      gsync();
      if (nw > 0) {
        for (int t = 0; t < jn; ++t) {
          const i64 j = j1 - t;
          const int xs = (int)(j - base);
          if (own) {
            const T xv = X[xs * nr + oc];
            if (is_nonzero(xv)) X[xs * nr + oc] = div_staged(xv, LC[t * (kv + 1)], RH[t], RH[kChunk + t]);
          }
          wsync();
          if (cok) {
            const T xj = X[xs * nr + cl];
            if (is_nonzero(xj)) {
              const T tt = -xj;
              const int lim = (int)min((i64)kv, j);
              for (int i = 1 + r0; i <= lim; i += rstep)
                X[(xs - i) * nr + cl] = fma(tt, LC[t * (kv + 1) + i], X[(xs - i) * nr + cl]);
            }
          }
          wsync();
        }
      }
      gsync();
      store_rows((int)(j1 - jn + 1 - base), (int)(j1 + 1 - base), base);
      gsync();
      j1 -= jn;
      if (j1 < 0) break;
      grp_shift_up<T, G>(X, (XW - jn) * nr, jn * nr);
      base -= jn;
      load_rows(0, jn, base);
      gsync();
    }
  } else {
    // ---- U^T y = b (dtbsv 'U','T','N') in axpy form: once x_i is final, x_c -= U(i,c) x_i
    load_rows(0, XW, 0);
    gsync();
    for (i64 j0 = 0; j0 < n; j0 += kCh) {
      const int jn = (int)min((i64)kCh, n - j0);
      // row i of U: U(i, i+c) = ab[(kv-c) + (i+c)*ldab], c = 0..kv
      for (int t = 0; t < jn; ++t) {
        const i64 i = j0 + t;
        for (int c = tid; c <= kv; c += NT)
          cp_async_elem(LC + t * (kv + 1) + c, i + c < n ? ab + (kv - c) + (i + c) * ldab : ab, i + c < n);
      }
      cp_async_commit();
      T* RH = reinterpret_cast<T*>(IP);
      for (int t = tid; t < jn; t += NT) div_rcp(ab[kv + (j0 + t) * ldab], RH[t], RH[kChunk + t]);
      cp_async_wait<0>();
      gsync();
      if (nw > 0) {
        for (int t = 0; t < jn; ++t) {
          const i64 i = j0 + t;
          if (own) X[t * nr + oc] = div_staged(X[t * nr + oc], LC[t * (kv + 1)], RH[t], RH[kChunk + t]);
          wsync();
          if (cok) {
            const T xi = X[t * nr + cl];
            const int lim = (int)min((i64)kv, n - 1 - i);
            for (int c = 1 + r0; c <= lim; c += rstep)
              X[(t + c) * nr + cl] = fma(-LC[t * (kv + 1) + c], xi, X[(t + c) * nr + cl]);
          }
          wsync();
        }
      }
      gsync();
      store_rows(0, jn, j0);
      gsync();
      grp_shift_down<T, G>(X, (XW - jn) * nr, jn * nr);
      load_rows(XW - jn, XW, j0 + jn);
      gsync();
    }
    // ---- L^T with interchanges, j = n-2 .. 0 (dgbtrs 'T': dgemv then dswap).  Chunk of
    // steps j = j1 .. j1-jn+1; window rows s <-> b rows base + s, base = j1-jn+1,
    // holding rows base .. j1+kl; after the chunk, rows above j1-jn+1+kl are final.
    if (kl > 0 && n > 1) {
      i64 j1 = n - 2;
      int jn = (int)min((i64)kCh, j1 + 1);
      i64 base = j1 - jn + 1;
      load_rows(0, jn + kl, base);
      while (true) {
        // LC[t][i] = L(j+1+i, j), j = j1 - t; IP[t] = pivot row of j, in the window
        for (int t = 0; t < jn; ++t) {
          const i64 j = j1 - t;
          for (int i = tid; i < kl; i += NT) cp_async_elem(LC + t * kl + i, ab + (kv + 1 + i) + j * ldab, j + 1 + i < n);
        }
        cp_async_commit();
        for (int t = tid; t < jn; t += NT) IP[t] = ipiv[j1 - t] - 1 - base;
        cp_async_wait<0>();
        gsync();
        if (nw > 0) {
          for (int t = 0; t < jn; ++t) {
            const i64 j = j1 - t;
            const int s0 = (int)(j - base);
            const int lm = (int)min((i64)kl, n - 1 - j);
            const T* lc = LC + t * kl;
            if (kl <= 16) {  // sequential fma dot product, as reference dgemv 'T'
              if (own) {
                T temp = T(0);
                for (int i = 0; i < lm; ++i) temp = fma(X[(s0 + 1 + i) * nr + oc], lc[i], temp);
                X[s0 * nr + oc] = fma(T(-1), temp, X[s0 * nr + oc]);
              }
            } else if (split) {  // group tree reduction per column (partials in the header)
              for (int c = 0; c < nr; ++c) {
                T temp = T(0);
                for (int i = tid; i < lm; i += NT) temp = fma(X[(s0 + 1 + i) * nr + c], lc[i], temp);
#pragma unroll
                for (int off = 16; off >= 1; off >>= 1) temp += __shfl_down_sync(0xffffffffu, temp, off);
                if (lane == 0) smem[8 + wig] = temp;
                Grp<G>::sync();
                if (wig == 0) {  // the warps' partials by a shuffle tree (log2 G dependent adds)
                  T sum = lane < G ? smem[8 + lane] : T(0);
#pragma unroll
                  for (int off = G / 2; off >= 1; off >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, off);
                  if (lane == 0) X[s0 * nr + c] = fma(T(-1), sum, X[s0 * nr + c]);
                }
                Grp<G>::sync();
              }
            } else {  // warp tree reduction per column
              for (int c = cw0; c < cw0 + nw; ++c) {
                T temp = T(0);
                for (int i = lane; i < lm; i += 32) temp = fma(X[(s0 + 1 + i) * nr + c], lc[i], temp);
#pragma unroll
                for (int off = 16; off >= 1; off >>= 1) temp += __shfl_down_sync(0xffffffffu, temp, off);
                if (lane == 0) X[s0 * nr + c] = fma(T(-1), temp, X[s0 * nr + c]);
              }
            }
            wsync();
            const int l = (int)IP[t];
            if (l != s0 && own) {
              const T tv = X[l * nr + oc];
              X[l * nr + oc] = X[s0 * nr + oc];
              X[s0 * nr + oc] = tv;
            }
            wsync();
          }
        }
        gsync();
        // rows base + jn - 1 + kl + 1 .. are final: window rows jn + kl - ... ; store the
        // window's top jn rows that are now final (s >= kl ... window end) and slide down
        const i64 nb = j1 - jn;  // next chunk's top step
        if (nb < 0) {
          store_rows(0, jn + kl, base);
          gsync();
          break;
        }
        const int jn2 = (int)min((i64)kCh, nb + 1);
        // final rows: b rows > base + kl - 1 + ... = rows base + kl .. base + jn + kl - 1
        // become final only after the steps they can still be swapped with; steps of the
        // next chunk touch rows <= nb + kl = base - 1 + kl, so rows base + kl .. are final
        store_rows(kl, jn + kl, base);
        gsync();
        grp_shift_up<T, G>(X, kl * nr, jn2 * nr);  // rows 0..kl-1 move to jn2..jn2+kl-1
        base = nb - jn2 + 1;
        j1 = nb;
        jn = jn2;
        load_rows(0, jn, base);
        gsync();
      }
    }
  }
}

// All nrhs right-hand sides, kMaxRhs per sweep.
template <typename T, int G>
__device__ void gbtrs_all(bool trans, i64 n, int kl, int ku, i64 nrhs, const T* __restrict__ ab, i64 ldab,
                          const i64* __restrict__ ipiv, T* __restrict__ b, i64 ldb, T* __restrict__ smem,
                          int ch = kChunk) {
  if (n <= 0) return;
  for (i64 c0 = 0; c0 < nrhs; c0 += kMaxRhs)
    gbtrs_group<T, G>(trans, n, kl, ku, (int)min((i64)kMaxRhs, nrhs - c0), ab, ldab, ipiv, b + c0 * ldb, ldb, smem,
                      ch);
}

}  // namespace bm
