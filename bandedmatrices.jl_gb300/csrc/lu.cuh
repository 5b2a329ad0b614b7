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
// into a staging ring.  The arithmetic is LAPACK's dgbtf2 operation for operation:
// idamax (first index of the largest |a|), row interchange over columns j..ju,
// scaling by the reciprocal of the pivot, and the rank-1 update a <- fma(l_i, -u_c, a)
// skipping u_c == 0 -- so factors and pivots equal the oracle's bit for bit.
//
// gbtrs: the sweeps are sequential in j; each step's update is spread over the
// group's threads, up to kMaxRhs right-hand sides at once, and b is staged through
// shared memory in chunks of kChunk steps.  Every element receives its updates in
// the same order as in dgbtrs/dtbsv (the transposed triangular solve is done in axpy
// form, which preserves each element's accumulation order).  Only the L^T dot
// products of the transposed solve use a tree reduction when kl > 16.
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

constexpr int kChunk = 32;  // solve steps staged per chunk
constexpr int kMaxRhs = 8;  // right-hand sides swept together
__host__ __device__ inline i64 gbtrs_smem_elems(int kl, int ku) {
  const int kv = kl + ku;
  // header + ipiv chunk (kChunk int64, as 2*kChunk T slots) + window of b
  // ((kChunk+kv+1) rows x kMaxRhs) + chunk of L or U columns (kChunk x (kv+1))
  return kHdr + 2 * kChunk + (i64)(kChunk + kv + 1) * kMaxRhs + (i64)kChunk * (kv + 1);
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

// --------------------------------------------------------------------- gbtrs
// Thread layout for a group of nr <= kMaxRhs right-hand sides: nr is padded to a
// power of two 1 << lg; thread -> (row offset tid >> lg, column tid & ((1<<lg)-1)),
// rows advancing by NT >> lg.  Window element (row s, column c) lives at X[s*nr + c].
__device__ __forceinline__ int rhs_lg(int nr) { return nr <= 1 ? 0 : nr <= 2 ? 1 : nr <= 4 ? 2 : 3; }

// Solves op(A) X = B for nr <= kMaxRhs right-hand sides (B: n x nr, leading dim ldb)
// with the gbtrf factors; trans: false = 'N', true = 'T'.
template <typename T, int G>
__device__ void gbtrs_group(bool trans, i64 n, int kl, int ku, int nr, const T* __restrict__ ab, i64 ldab,
                            const i64* __restrict__ ipiv, T* __restrict__ b, i64 ldb, T* __restrict__ smem) {
  constexpr int NT = Grp<G>::NT;
  const int tid = Grp<G>::tid(), lane = threadIdx.x & 31, wig = tid >> 5;
  const int kv = kl + ku;
  const int lg = rhs_lg(nr), cl = tid & ((1 << lg) - 1), rstep = NT >> lg, r0 = tid >> lg;
  const bool cok = cl < nr;
  i64* IP = reinterpret_cast<i64*>(smem + kHdr);  // kChunk pivots (8-byte aligned)
  T* X = smem + kHdr + 2 * kChunk;                // window: XW rows x nr
  const int XW = kChunk + kv + 1;
  T* LC = X + XW * kMaxRhs;                       // kChunk columns x (kv+1)
  auto sync = [] { Grp<G>::sync(); };
  // copy window rows [s0, s1) from/to b rows [g0 + s0, ...), zero outside [0, n)
  auto load_rows = [&](int s0, int s1, i64 g0) {
    for (int sr = s0 + r0; sr < s1; sr += rstep)
      if (cok) X[sr * nr + cl] = (g0 + sr >= 0 && g0 + sr < n) ? b[(g0 + sr) + cl * ldb] : T(0);
  };
  auto store_rows = [&](int s0, int s1, i64 g0) {
    for (int sr = s0 + r0; sr < s1; sr += rstep)
      if (cok && g0 + sr >= 0 && g0 + sr < n) b[(g0 + sr) + cl * ldb] = X[sr * nr + cl];
  };

  if (!trans) {
    // ---- forward: L with row interchanges (dgbtrs 'N': dswap + dger per column)
    if (kl > 0 && n > 1) {
      load_rows(0, kl, 0);
      for (i64 j0 = 0; j0 < n - 1; j0 += kChunk) {
        const int jn = (int)min((i64)kChunk, n - 1 - j0);
        load_rows(kl, jn + kl, j0);
        for (int e = tid; e < jn * kl; e += NT) {
          const int sidx = e / kl, i = e - sidx * kl;
          LC[sidx * kl + i] = (j0 + sidx + 1 + i < n) ? ab[(kv + 1 + i) + (j0 + sidx) * ldab] : T(0);
        }
        for (int sidx = tid; sidx < jn; sidx += NT) IP[sidx] = ipiv[j0 + sidx] - 1 - j0;
        sync();
        for (int st = 0; st < jn; ++st) {
          const int lm = (int)min((i64)kl, n - 1 - (j0 + st));
          const int l = (int)IP[st];
          if (l != st) {
            if (tid < nr) {
              const T t = X[l * nr + tid];
              X[l * nr + tid] = X[st * nr + tid];
              X[st * nr + tid] = t;
            }
            sync();
          }
          if (cok) {
            const T bj = X[st * nr + cl];
            if (bj != T(0)) {
              const T t = -bj;
              for (int i = r0; i < lm; i += rstep)
                X[(st + 1 + i) * nr + cl] = fma(LC[st * kl + i], t, X[(st + 1 + i) * nr + cl]);
            }
          }
          sync();
        }
        store_rows(0, jn, j0);
        sync();
        grp_shift_down<T, G>(X, kl * nr, jn * nr);  // carry rows jn .. jn+kl to the front
        if (j0 + jn >= n - 1) store_rows(0, kl, j0 + jn);
        sync();
      }
    }
    // ---- backward: U x = y (dtbsv 'U','N','N', bandwidth kv), columns n-1 .. 0;
    // window row s <-> b row base + s, with row XW-1 = j1 at the start of each chunk
    i64 j1 = n - 1;
    i64 base = j1 - (XW - 1);
    load_rows(0, XW, base);
    sync();
    while (true) {
      const int jn = (int)min((i64)kChunk, j1 + 1);
      // U(j-i, j) = ab[(kv-i) + j*ldab], i = 0..kv, for j = j1, j1-1, ...
      for (int e = tid; e < jn * (kv + 1); e += NT) {
        const int t = e / (kv + 1), i = e - t * (kv + 1);
        const i64 j = j1 - t;
        LC[e] = (j - i >= 0) ? ab[(kv - i) + j * ldab] : T(0);
      }
      sync();
      for (int t = 0; t < jn; ++t) {
        const i64 j = j1 - t;
        const int xs = (int)(j - base);
        if (tid < nr) {
          const T xv = X[xs * nr + tid];
          if (xv != T(0)) X[xs * nr + tid] = xv / LC[t * (kv + 1)];
        }
        sync();
        if (cok) {
          const T xj = X[xs * nr + cl];
          if (xj != T(0)) {
            const T tt = -xj;
            const int lim = (int)min((i64)kv, j);
            for (int i = 1 + r0; i <= lim; i += rstep)
              X[(xs - i) * nr + cl] = fma(tt, LC[t * (kv + 1) + i], X[(xs - i) * nr + cl]);
          }
        }
        sync();
      }
      store_rows((int)(j1 - jn + 1 - base), (int)(j1 + 1 - base), base);
      sync();
      j1 -= jn;
      if (j1 < 0) break;
      grp_shift_up<T, G>(X, (XW - jn) * nr, jn * nr);
      base -= jn;
      load_rows(0, jn, base);
      sync();
    }
  } else {
    // ---- U^T y = b (dtbsv 'U','T','N') in axpy form: once x_i is final, x_c -= U(i,c) x_i
    load_rows(0, XW, 0);
    sync();
    for (i64 j0 = 0; j0 < n; j0 += kChunk) {
      const int jn = (int)min((i64)kChunk, n - j0);
      // row i of U: U(i, i+c) = ab[(kv-c) + (i+c)*ldab], c = 0..kv
      for (int e = tid; e < jn * (kv + 1); e += NT) {
        const int t = e / (kv + 1), c = e - t * (kv + 1);
        const i64 i = j0 + t;
        LC[e] = (i + c < n) ? ab[(kv - c) + (i + c) * ldab] : T(0);
      }
      sync();
      for (int t = 0; t < jn; ++t) {
        const i64 i = j0 + t;
        if (tid < nr) X[t * nr + tid] = X[t * nr + tid] / LC[t * (kv + 1)];
        sync();
        if (cok) {
          const T xi = X[t * nr + cl];
          const int lim = (int)min((i64)kv, n - 1 - i);
          for (int c = 1 + r0; c <= lim; c += rstep)
            X[(t + c) * nr + cl] = fma(-LC[t * (kv + 1) + c], xi, X[(t + c) * nr + cl]);
        }
        sync();
      }
      store_rows(0, jn, j0);
      sync();
      grp_shift_down<T, G>(X, (XW - jn) * nr, jn * nr);
      load_rows(XW - jn, XW, j0 + jn);
      sync();
    }
    // ---- L^T with interchanges, j = n-2 .. 0 (dgbtrs 'T': dgemv then dswap)
    if (kl > 0) {
      for (i64 j = n - 2; j >= 0; --j) {
        const int lm = (int)min((i64)kl, n - 1 - j);
        const T* lc = ab + (kv + 1) + j * ldab;
        if (kl <= 16) {
          if (tid < nr) {
            T temp = T(0);
            for (int i = 0; i < lm; ++i) temp = fma(b[(j + 1 + i) + tid * ldb], lc[i], temp);
            b[j + tid * ldb] = fma(T(-1), temp, b[j + tid * ldb]);
          }
        } else if (wig == 0) {
          for (int c = 0; c < nr; ++c) {
            T temp = T(0);
            for (int i = lane; i < lm; i += 32) temp = fma(b[(j + 1 + i) + c * ldb], lc[i], temp);
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) temp += __shfl_down_sync(0xffffffffu, temp, off);
            if (lane == 0) b[j + c * ldb] = fma(T(-1), temp, b[j + c * ldb]);
          }
        }
        __threadfence_block();
        sync();
        const i64 l = ipiv[j] - 1;
        if (l != j && tid < nr) {
          const T t = b[l + tid * ldb];
          b[l + tid * ldb] = b[j + tid * ldb];
          b[j + tid * ldb] = t;
        }
        __threadfence_block();
        sync();
      }
    }
  }
}

// All nrhs right-hand sides, kMaxRhs per sweep.
template <typename T, int G>
__device__ void gbtrs_all(bool trans, i64 n, int kl, int ku, i64 nrhs, const T* __restrict__ ab, i64 ldab,
                          const i64* __restrict__ ipiv, T* __restrict__ b, i64 ldb, T* __restrict__ smem) {
  if (n <= 0) return;
  for (i64 c0 = 0; c0 < nrhs; c0 += kMaxRhs)
    gbtrs_group<T, G>(trans, n, kl, ku, (int)min((i64)kMaxRhs, nrhs - c0), ab, ldab, ipiv, b + c0 * ldb, ldb, smem);
}

}  // namespace bm
