// gbmm: C <- alpha*A*B + beta*C for banded A (n x nu, (Al,Au)), B (nu x m, (Bl,Bu)) and
// C (n x m, (Cl,Cu)) whose band holds every in-matrix nonzero of A*B (Cl >= min(Al+Bl, n-1),
// Cu >= min(Au+Bu, m-1)), all in LAPACK band storage.
//
// Replaces gbmm!/_gbmm! (src/banded/gbmm.jl:207-340), which computes every column of C
// as one small dgbmv over a window of A; the arithmetic is banded_mul!
// (src/generic/matmul.jl:143-172).  Each C entry is accumulated exactly as that column
// dgbmv does: c = beta*c, then c = fma(alpha*B(v,j), A(k,v), c) for v ascending over
// max(0,k-Al,j-Bu) <= v <= min(nu-1,k+Au,j+Bl).  Bands of C outside (Al+Bl, Au+Bu) are
// scaled by beta (set to zero when beta == 0, C not read), as gbmm! does (:286-288).
//
// Three paths, all in that order:
//   * interior column tiles with beta == 0 and bands of at most 33 rows take a
//     register-blocked kernel: gbmm_f32x2_kernel (Float32: TMA bulk tiles, packed fma
//     pairs) or gbmm_reg_kernel (Float64, or Float32 with an even lda);
//   * the edge columns of those shapes take gbmm_simple_kernel (a thread per entry);
//   * everything else takes gbmm_tma_kernel: a persistent kernel over tiles of TJ C
//     columns, whose thread 0 streams A's columns [j0-Bu, j0+TJ+Bl), B's columns and
//     (beta != 0) C's columns into a two-slot ring with 1-D TMA bulk copies, a warp per
//     C column and its lanes over the column's storage rows.
// Roofline: HBM for Float32; the FP64 pipe for Float64 on GB300 (about 2 flop/byte).
#include <cstdio>
#include <cstdlib>

#include "common.cuh"

namespace bm {

template <typename T>
struct GbmmParams {
  i64 n, nu, m;
  int Al, Au, Bl, Bu, Cl, Cu;
  i64 lda, ldb, ldc;
  T alpha, beta;
  const T* A;
  const T* B;
  T* C;
  i64 tile, ntiles;
  i64 jskip0, jskip1;  // columns [jskip0, jskip1) are written by the interior kernel
  int stages;
  uint32_t stage_bytes, boff, coff;
  int* status;
};

struct Span {
  i64 gs, ge, end;  // first element in smem (16-byte rounded), end of bulk part, end
};

template <typename T>
__device__ __forceinline__ Span span_of(i64 start, i64 end) {
  constexpr i64 q = 16 / sizeof(T);
  Span r;
  if (end <= start) {
    r.gs = r.ge = r.end = start & ~(q - 1);
    return r;
  }
  r.gs = start & ~(q - 1);
  r.ge = end & ~(q - 1);
  if (r.ge < r.gs) r.ge = r.gs;
  r.end = end;
  return r;
}

template <typename T>
__device__ __forceinline__ void gbmm_tile(const GbmmParams<T>& p, i64 t, i64& j0, i64& j1, i64& a0, i64& a1) {
  j0 = t * p.tile;
  j1 = min(j0 + p.tile, p.m);
  a0 = max((i64)0, j0 - p.Bu);
  a1 = min(p.nu, j1 + p.Bl);
  if (a1 < a0) a1 = a0;
}

template <typename T>
__device__ __forceinline__ void gbmm_issue(const GbmmParams<T>& p, unsigned char* slots, uint64_t* bars, i64 k) {
  const i64 t = (i64)blockIdx.x + k * (i64)gridDim.x;
  if (t >= p.ntiles) return;
  const int s = (int)(k % p.stages);
  i64 j0, j1, a0, a1;
  gbmm_tile(p, t, j0, j1, a0, a1);
  const Span sa = span_of<T>(a0 * p.lda, a1 * p.lda);
  const Span sb = span_of<T>(j0 * p.ldb, j1 * p.ldb);
  const Span sc = (p.beta != T(0)) ? span_of<T>(j0 * p.ldc, j1 * p.ldc) : span_of<T>(0, 0);
  const uint32_t ba = (uint32_t)((sa.ge - sa.gs) * (i64)sizeof(T));
  const uint32_t bb = (uint32_t)((sb.ge - sb.gs) * (i64)sizeof(T));
  const uint32_t bc = (uint32_t)((sc.ge - sc.gs) * (i64)sizeof(T));
  unsigned char* slot = slots + (size_t)s * p.stage_bytes;
  fence_proxy_async_smem();
  mbar_arrive_expect_tx(&bars[s], ba + bb + bc);
  if (ba) bulk_g2s(slot, p.A + sa.gs, ba, &bars[s]);
  if (bb) bulk_g2s(slot + p.boff, p.B + sb.gs, bb, &bars[s]);
  if (bc) bulk_g2s(slot + p.coff, p.C + sc.gs, bc, &bars[s]);
}

// Up to kSlots*32 C storage rows per column (Cl+Cu+1 <= 32*kSlots).
template <typename T, int kSlots>
__global__ void __launch_bounds__(256) gbmm_tma_kernel(const GbmmParams<T> p) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  unsigned char* slots = smem + 128;
  if (threadIdx.x == 0) {
    for (int s = 0; s < p.stages; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = 0; k < p.stages; ++k) gbmm_issue(p, slots, bars, k);

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int crows = p.Cl + p.Cu + 1;
  const int ka = p.Al + p.Au;                    // last A storage row
  const int kbmax = p.Bl + p.Bu;                 // last B storage row
  const int lda = (int)p.lda, ldb = (int)p.ldb, ldc = (int)p.ldc;
  i64 k = 0;
  bool failed = false;
  for (;; ++k) {
    const i64 t = (i64)blockIdx.x + k * (i64)gridDim.x;
    if (t >= p.ntiles) break;
    const int s = (int)(k % p.stages);
    const bool ok = mbar_wait(&bars[s], (uint32_t)((k / p.stages) & 1));
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    i64 j0, j1, a0, a1;
    gbmm_tile(p, t, j0, j1, a0, a1);
    const Span sa = span_of<T>(a0 * p.lda, a1 * p.lda);
    const Span sb = span_of<T>(j0 * p.ldb, j1 * p.ldb);
    const bool usec = p.beta != T(0);
    const Span sc = usec ? span_of<T>(j0 * p.ldc, j1 * p.ldc) : span_of<T>(0, 0);
    T* As = reinterpret_cast<T*>(slots + (size_t)s * p.stage_bytes);
    T* Bs = reinterpret_cast<T*>(slots + (size_t)s * p.stage_bytes + p.boff);
    T* Cs = reinterpret_cast<T*>(slots + (size_t)s * p.stage_bytes + p.coff);
    {  // ragged tails (< 16 bytes) the bulk copies left out
      const int tid = threadIdx.x;
      const int na = (int)(sa.end - sa.ge), nb = (int)(sb.end - sb.ge), nc = (int)(sc.end - sc.ge);
      if (tid < na) As[sa.ge - sa.gs + tid] = p.A[sa.ge + tid];
      else if (tid >= 32 && tid - 32 < nb) Bs[sb.ge - sb.gs + tid - 32] = p.B[sb.ge + tid - 32];
      else if (tid >= 64 && tid - 64 < nc) Cs[sc.ge - sc.gs + tid - 64] = p.C[sc.ge + tid - 64];
    }
    if (p.alpha != T(1)) {  // B <- alpha*B once per tile (the column dgbmv's temp = alpha*x)
      __syncthreads();
      const i64 cnt = (j1 - j0) * p.ldb;
      for (i64 e = threadIdx.x; e < cnt; e += blockDim.x) {
        T* q = Bs + (j0 * p.ldb - sb.gs) + e;
        *q = p.alpha * *q;
      }
    }
    __syncthreads();

    const int abase = (int)(a0 * p.lda - sa.gs);
    const int bbase = (int)(j0 * p.ldb - sb.gs);
    const int cbase = (int)(j0 * p.ldc - sc.gs);
    for (i64 j = j0 + warp; j < j1; j += nwarps) {
      const int jl = (int)(j - j0);
      // terms rb = v - (j - Bu) in [rb_lo, rb_hi]: B's band intersected with 0 <= v < nu
      const int rb_lo = (int)max((i64)0, p.Bu - j);
      const int rb_hi = (int)min((i64)kbmax, p.nu - 1 - j + p.Bu);
      T acc[kSlots];
      int rcs[kSlots];
      bool live[kSlots];  // an in-matrix entry of C's band
#pragma unroll
      for (int q = 0; q < kSlots; ++q) {
        const int rc = lane + 32 * q;
        rcs[q] = rc;
        const i64 row = j + rc - p.Cu;
        live[q] = rc < crows && row >= 0 && row < p.n;
        acc[q] = (usec && live[q]) ? p.beta * Cs[cbase + jl * ldc + rc] : T(0);
      }
      // A(k,v) with k = j + rc - Cu, v = j - Bu + rb:  storage row ra = Au + k - v
      //   = rc - rb + (Au + Bu - Cu);  smem column offset (v - a0)
      const int shift = p.Au + p.Bu - p.Cu;
      for (int rb = rb_lo; rb <= rb_hi; ++rb) {
        const T b = Bs[bbase + jl * ldb + rb];
        const int vcol = (int)(j - p.Bu + rb - a0);
        const T* acol = As + abase + vcol * lda;
#pragma unroll
        for (int q = 0; q < kSlots; ++q) {
          const int ra = rcs[q] - rb + shift;
          if (live[q] && ra >= 0 && ra <= ka) acc[q] = fma(b, acol[ra], acc[q]);
        }
      }
      // write in-matrix entries; bands outside the product get beta*C (0 if beta == 0)
#pragma unroll
      for (int q = 0; q < kSlots; ++q)
        if (live[q]) p.C[j * p.ldc + rcs[q]] = acc[q];
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) gbmm_issue(p, slots, bars, k + p.stages);
  }
  if (failed) {
    if (threadIdx.x == 0) record_status(p.status, BM_STATUS_TIMEOUT);
    for (i64 kk = k; kk < k + p.stages; ++kk) {
      const i64 t = (i64)blockIdx.x + kk * (i64)gridDim.x;
      if (t >= p.ntiles) break;
      (void)mbar_wait(&bars[kk % p.stages], (uint32_t)((kk / p.stages) & 1));
    }
  }
}

// ---------------------------------------------------------------- interior tiles
// Columns j whose every term lies inside the matrices (Au+Bu <= j, j+Bl < nu,
// j+Al+Bl < n) take a register-blocked path when beta == 0 and both bands have at most
// MA = MB rows (a size class: 9, 17 or 33).  A thread owns CPT consecutive C columns
// and keeps their product bands (NA+NB-1 entries each, NA = Al+Au+1, NB = Bl+Bu+1) in
// registers.  The outer loop walks A's columns v ascending (for column j the B band
// row is ob = v - j + Bu), the inner loop A's rows ra; entry ra+ob of the column
// receives fma(alpha*B(v,j), A(ra,v), .).  Every C entry therefore gets its terms in
// ascending v from a zero start: the same fma chain as the column dgbmv of _gbmm!.
// Both loops are unrolled, so the accumulator index is a compile-time register.
//
// A's window and B's columns are staged in shared memory at odd strides (SA = NA|1,
// SB = NB|1); for CPT == 2 the columns are split by parity into two halves, so lane t
// (columns 2t, 2t+1, window columns 2t+ob) reads address t*SA + const: 32 distinct
// banks for 4- and 8-byte elements.  One A load feeds CPT fmas.  The product goes
// back through shared memory (stride SC = (NA+NB-1)|1) for coalesced stores.
// Bound: HBM for Float32 (about 2 instructions per fma); the FP64 pipe for Float64.
constexpr int kRegNT = 128;

struct FastDiv {  // x / d for x < 2^32 by multiply-high (round-up method, Granlund-Montgomery)
  uint32_t mul;
  int shift;
};
static FastDiv make_fastdiv(uint32_t d) {
  FastDiv f;
  int s = 0;
  while ((1ull << s) < d) ++s;
  f.shift = s;
  f.mul = (uint32_t)(((((uint64_t)1 << s) - d) << 32) / d + 1);
  return f;
}
__device__ __forceinline__ uint32_t fdiv(uint32_t x, const FastDiv f) {
  return (uint32_t)(((uint64_t)__umulhi(x, f.mul) + x) >> f.shift);
}

struct RegTile {
  int NA, NB, rows_prod, shift;  // shift = Cu - (Au + Bu): C row of product entry 0
  uint32_t SA, SB, SC;           // odd shared-memory strides
  uint32_t ahalf, bhalf, chalf;  // offsets of the odd-column halves (CPT == 2)
  uint32_t boff;                 // offset of the B tile
  i64 F0, ntiles;                // first column of tile 0, number of tiles
  FastDiv dlda, dldb, dldc;
};

template <int CPT>
__device__ __forceinline__ uint32_t col_off(uint32_t c, uint32_t S, uint32_t half) {
  if constexpr (CPT == 1) return c * S;
  else return (c & 1u) * half + (c >> 1) * S;
}

template <typename T, int MA, int MB, int CPT, bool EXACT>
__device__ __forceinline__ void reg_columns(const RegTile& rt, const T alpha, const T* __restrict__ As,
                                            const T* __restrict__ Bs, T (&acc)[CPT][MA + MB - 1]) {
  const uint32_t t = threadIdx.x;
  const int NA = rt.NA, NB = rt.NB;
  const bool scale = alpha != T(1);
  const T* bcol[CPT];
#pragma unroll
  for (int q = 0; q < CPT; ++q) bcol[q] = Bs + col_off<CPT>(CPT * t + q, rt.SB, rt.bhalf);
#pragma unroll
  for (int ob = 0; ob < MB + CPT - 1; ++ob) {
    if (ob >= NB + CPT - 1) break;
    const T* ap = As + col_off<CPT>(CPT * t + ob, rt.SA, rt.ahalf);
    T b[CPT];
    bool use[CPT];
#pragma unroll
    for (int q = 0; q < CPT; ++q) {
      const int rb = ob - q;  // B band row of column CPT*t + q
      use[q] = rb >= 0 && rb < MB && rb < NB;
      const T bv = use[q] ? bcol[q][rb] : T(0);
      b[q] = scale ? alpha * bv : bv;  // the column dgbmv's temp = alpha*x
    }
#pragma unroll
    for (int ra = 0; ra < MA; ++ra) {
      if (!EXACT && ra >= NA) break;
      const T a = ap[ra];
#pragma unroll
      for (int q = 0; q < CPT; ++q)
        if (ob - q >= 0 && ob - q < MB && use[q]) acc[q][ra + ob - q] = fma(b[q], a, acc[q][ra + ob - q]);
    }
  }
}

template <typename T, int MA, int MB, int CPT>
__global__ void __launch_bounds__(kRegNT, sizeof(T) == 4 ? 3 : 2) gbmm_reg_kernel(const GbmmParams<T> p, const RegTile rt) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  constexpr int TJ = kRegNT * CPT;
  constexpr int NP = MA + MB - 1;
  const uint32_t t = threadIdx.x;
  const int NA = rt.NA, NB = rt.NB;
  const uint32_t lda = (uint32_t)p.lda, ldb = (uint32_t)p.ldb, ldc = (uint32_t)p.ldc;
  const int crows = p.Cl + p.Cu + 1;
  T* As = sm;
  T* Bs = sm + rt.boff;
  T* Cs = sm;  // the product reuses the A/B space
  for (i64 tile = blockIdx.x; tile < rt.ntiles; tile += gridDim.x) {
    const i64 j0 = rt.F0 + tile * TJ;
    const i64 v0 = j0 - p.Bu;
    // A's columns v0 .. v0+TJ+NB-2 (rows 0..NA-1) and B's columns j0 .. j0+TJ-1, one
    // cp.async per element: a thread issues all of its copies before waiting, so each
    // CTA keeps tens of KB in flight
    {
      const T* src = p.A + v0 * p.lda;
      const uint32_t cnt = (uint32_t)(TJ + NB - 1) * lda;
      for (uint32_t e = t; e < cnt; e += kRegNT) {
        const uint32_t c = fdiv(e, rt.dlda), r = e - c * lda;
        if (r < (uint32_t)NA) cp_async_elem(As + col_off<CPT>(c, rt.SA, rt.ahalf) + r, src + e, true);
      }
    }
    {
      const T* src = p.B + j0 * p.ldb;
      const uint32_t cnt = (uint32_t)TJ * ldb;
      for (uint32_t e = t; e < cnt; e += kRegNT) {
        const uint32_t c = fdiv(e, rt.dldb), r = e - c * ldb;
        if (r < (uint32_t)NB) cp_async_elem(Bs + col_off<CPT>(c, rt.SB, rt.bhalf) + r, src + e, true);
      }
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    T acc[CPT][NP];
#pragma unroll
    for (int q = 0; q < CPT; ++q)
#pragma unroll
      for (int i = 0; i < NP; ++i) acc[q][i] = T(0);
    if (NA == MA) reg_columns<T, MA, MB, CPT, true>(rt, p.alpha, As, Bs, acc);
    else reg_columns<T, MA, MB, CPT, false>(rt, p.alpha, As, Bs, acc);
    __syncthreads();  // every read of the A/B tiles is done
#pragma unroll
    for (int q = 0; q < CPT; ++q) {
      T* cc = Cs + col_off<CPT>(CPT * t + q, rt.SC, rt.chalf);
#pragma unroll
      for (int i = 0; i < NP; ++i)
        if (i < rt.rows_prod) cc[i] = acc[q][i];
    }
    __syncthreads();
    {  // columns j0 .. j0+TJ-1 of C: product rows, and zeros in the other in-matrix rows
      T* dst = p.C + j0 * p.ldc;
      const uint32_t cnt = (uint32_t)TJ * ldc;
      for (uint32_t e = t; e < cnt; e += kRegNT) {
        const uint32_t c = fdiv(e, rt.dldc);
        const int r = (int)(e - c * ldc);
        const int i = r - rt.shift;
        if (i >= 0 && i < rt.rows_prod) {
          dst[e] = Cs[col_off<CPT>(c, rt.SC, rt.chalf) + i];
        } else if (r < crows) {
          const i64 k = j0 + c + r - p.Cu;
          if (k >= 0 && k < p.n) dst[e] = T(0);
        }
      }
    }
    __syncthreads();  // the staged product is consumed before the next tile's loads
  }
}

// ------------------------------------------ Float32 interior tiles, packed fmas, TMA
// The Float32 interior path when A's leading dimension is odd, C has no padding rows
// (ldc == Cl+Cu+1) and every operand is 16-byte aligned.  The A, B and C tiles move as
// 1-D TMA bulk copies in their band-storage layouts, so no thread spends instructions
// on staging, and the inner loop reads A two rows at a time.  Lane t owns columns 2t
// and 2t+1; its window column at step ob is 2t+ob, whose shared-memory start has the
// parity of ob (lda odd, every tile starts at an even window column), so rows (r, r+1)
// with r = ob mod 2 are an aligned 8-byte pair.  A 64-bit shared load is served per
// half-warp, and lanes t = 0..15 sit 8*lda bytes apart (lda odd): 16 distinct bank
// pairs.  Each pair feeds two packed fmas (__ffma2_rn, per component identical to
// fmaf): (acc0[k], acc0[k+1]) += b0*(a_r, a_r+1) for column 2t and (acc1[k-1], acc1[k])
// += b1*(a_r, a_r+1) for column 2t+1, k = r + ob.  So the accumulator pairs are fixed
// registers (acc0 pairs start at even entries, acc1 pairs at odd ones), and every C
// entry still gets one term per step in ascending ob.
constexpr int kX2NT = 128;
constexpr int kX2TJ = 2 * kX2NT;

struct X2Tile {
  int NA, NB, NP, shift;  // NP = NA+NB-1 product rows; shift = C row of product entry 0
  i64 F0, ntiles;
  uint32_t a_elems;  // floats reserved for the A tile (a multiple of 4)
};

// entry m of column 2t (P0 pairs (2i, 2i+1)) and of column 2t+1 (P1 pairs (2i-1, 2i))
template <int N>
__device__ __forceinline__ float& acc0_at(float2 (&P0)[N], int m) {
  return (m & 1) ? P0[m >> 1].y : P0[m >> 1].x;
}
template <int N>
__device__ __forceinline__ float& acc1_at(float2 (&P1)[N], int m) {
  return (m & 1) ? P1[(m + 1) >> 1].x : P1[m >> 1].y;
}

template <int MA, int MB, bool EXACT>
__device__ __forceinline__ void x2_columns(int NA, int NB, float alpha, const float* __restrict__ As, int lda,
                                           const float* __restrict__ Bs, int ldb, float2 (&P0)[(MA + MB) / 2],
                                           float2 (&P1)[(MA + MB + 1) / 2]) {
  const int t = threadIdx.x;
  const bool scale = alpha != 1.f;
  const float* b0p = Bs + 2 * t * ldb;  // B column 2t
  const float* b1p = b0p + ldb;         // B column 2t+1
#pragma unroll
  for (int ob = 0; ob <= MB; ++ob) {
    if (ob > NB) break;
    const bool use0 = ob < MB && ob < NB;  // column 2t takes B rows 0..NB-1 at ob = 0..NB-1
    const bool use1 = ob >= 1;             // column 2t+1 takes them at ob = 1..NB
    float b0 = 0.f, b1 = 0.f;
    if (use0) b0 = scale ? alpha * b0p[ob] : b0p[ob];
    if (use1) b1 = scale ? alpha * b1p[ob - 1] : b1p[ob - 1];
    const float2 bb0 = make_float2(b0, b0), bb1 = make_float2(b1, b1);
    const float* ap = As + (2 * t + ob) * lda;
    if (ob & 1) {  // row 0 alone (the aligned pairs start at row 1)
      const float a = ap[0];
      if (use0) acc0_at(P0, ob) = fmaf(b0, a, acc0_at(P0, ob));
      acc1_at(P1, ob - 1) = fmaf(b1, a, acc1_at(P1, ob - 1));
    }
#pragma unroll
    for (int r = ob & 1; r < MA; r += 2) {
      const int k = r + ob;
      const bool pair = r + 1 < MA && (EXACT || r + 1 < NA);
      const bool last = !pair && (EXACT || r < NA);  // the last row alone
      if (pair) {
        const float2 pr = *reinterpret_cast<const float2*>(ap + r);
        if (use0) P0[k >> 1] = __ffma2_rn(pr, bb0, P0[k >> 1]);
        if (use1) P1[k >> 1] = __ffma2_rn(pr, bb1, P1[k >> 1]);
      } else if (last) {
        const float a = ap[r];
        if (use0) acc0_at(P0, k) = fmaf(b0, a, acc0_at(P0, k));
        if (use1) acc1_at(P1, k - 1) = fmaf(b1, a, acc1_at(P1, k - 1));
      }
    }
  }
}

template <int MA, int MB>
__global__ void __launch_bounds__(kX2NT, 3) gbmm_f32x2_kernel(const GbmmParams<float> p, const X2Tile xt) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  float* Araw = reinterpret_cast<float*>(smem_raw + 128);
  float* Braw = Araw + xt.a_elems;
  float* Craw = Araw;  // the product reuses the A/B space
  const int t = threadIdx.x;
  const int lda = (int)p.lda, ldb = (int)p.ldb, ldc = (int)p.ldc;
  const int crows = p.Cl + p.Cu + 1;
  const int nva = kX2TJ + xt.NB - 1;
  if (t == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  uint32_t phase = 0;
  for (i64 tile = blockIdx.x; tile < xt.ntiles; tile += gridDim.x, phase ^= 1u) {
    const i64 j0 = xt.F0 + tile * kX2TJ;
    const i64 v0 = j0 - p.Bu;
    // element ranges and their 16-byte-aligned starts; element e of a range sits at
    // [e - aligned start] in shared memory (the same 16-byte phase as in global memory)
    const i64 ea0 = v0 * p.lda, ea1 = (v0 + nva) * p.lda, ga0 = ea0 & ~3ll, ga1 = ea1 & ~3ll;
    const i64 eb0 = j0 * p.ldb, eb1 = (j0 + kX2TJ) * p.ldb, gb0 = eb0 & ~3ll, gb1 = eb1 & ~3ll;
    if (t == 0) {
      fence_proxy_async_smem();
      const uint32_t ba = (uint32_t)((ga1 - ga0) * 4), bb = (uint32_t)((gb1 - gb0) * 4);
      mbar_arrive_expect_tx(bar, ba + bb);
      if (ba) bulk_g2s(Araw, p.A + ga0, ba, bar);
      if (bb) bulk_g2s(Braw, p.B + gb0, bb, bar);
    } else if (t < 5) {  // up to three trailing elements past the last 16-byte boundary
      const i64 e = ga1 + t - 1;
      if (e >= ea0 && e < ea1) Araw[e - ga0] = p.A[e];
    } else if (t < 9) {
      const i64 e = gb1 + t - 5;
      if (e >= eb0 && e < eb1) Braw[e - gb0] = p.B[e];
    }
    const bool ok = mbar_wait(bar, phase);
    if (__syncthreads_or(!ok)) {
      if (t == 0) record_status(p.status, BM_STATUS_TIMEOUT);
      (void)mbar_wait(bar, phase);
      return;
    }
    float2 P0[(MA + MB) / 2], P1[(MA + MB + 1) / 2];
#pragma unroll
    for (int i = 0; i < (MA + MB) / 2; ++i) P0[i] = make_float2(0.f, 0.f);
#pragma unroll
    for (int i = 0; i < (MA + MB + 1) / 2; ++i) P1[i] = make_float2(0.f, 0.f);
    const float* As = Araw + (ea0 - ga0);
    const float* Bs = Braw + (eb0 - gb0);
    if (xt.NA == MA) x2_columns<MA, MB, true>(xt.NA, xt.NB, p.alpha, As, lda, Bs, ldb, P0, P1);
    else x2_columns<MA, MB, false>(xt.NA, xt.NB, p.alpha, As, lda, Bs, ldb, P0, P1);
    __syncthreads();  // every read of the A/B tiles is done
    const i64 ec0 = j0 * p.ldc, ec1 = (j0 + kX2TJ) * p.ldc, gc0 = ec0 & ~3ll;
    float* Cs = Craw + (ec0 - gc0);
    {
      float* c0 = Cs + 2 * t * ldc;
      float* c1 = c0 + ldc;
#pragma unroll
      for (int i = 0; i < MA + MB - 1; ++i)
        if (i < xt.NP) {
          c0[xt.shift + i] = acc0_at(P0, i);
          c1[xt.shift + i] = acc1_at(P1, i);
        }
      for (int r = 0; r < crows; ++r)  // C's bands outside the product: zero (beta == 0)
        if (r < xt.shift || r >= xt.shift + xt.NP) {
          c0[r] = 0.f;
          c1[r] = 0.f;
        }
    }
    fence_proxy_async_smem();
    __syncthreads();
    const i64 hc0 = (ec0 + 3) & ~3ll, hc1 = ec1 & ~3ll;  // the 16-byte-aligned middle
    if (t == 0) {
      bulk_s2g(p.C + hc0, Craw + (hc0 - gc0), (uint32_t)((hc1 - hc0) * 4));
      bulk_commit();
    } else if (t < 5) {
      const i64 e = ec0 + t - 1;
      if (e < hc0) p.C[e] = Craw[e - gc0];
    } else if (t < 9) {
      const i64 e = hc1 + t - 5;
      if (e < ec1) p.C[e] = Craw[e - gc0];
    }
    if (t == 0) bulk_wait_read_all();
    __syncthreads();  // the staged product is read before the next tile's copies land
  }
  if (t == 0) bulk_wait_all();
}

// Generic fallback (any alignment, very wide bands): one thread per C entry.
template <typename T>
__global__ void gbmm_simple_kernel(const GbmmParams<T> p) {
  const int crows = p.Cl + p.Cu + 1;
  const i64 skip = p.jskip1 - p.jskip0;
  const i64 total = (p.m - skip) * (i64)crows;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
    i64 j = e / crows;
    const int rc = (int)(e - j * crows);
    if (j >= p.jskip0) j += skip;
    const i64 row = j + rc - p.Cu;
    if (row < 0 || row >= p.n) continue;
    T acc = (p.beta == T(0)) ? T(0) : p.beta * p.C[j * p.ldc + rc];
    const i64 v0 = max(max((i64)0, row - p.Al), j - p.Bu);
    const i64 v1 = min(min(p.nu - 1, row + p.Au), j + p.Bl);
    for (i64 v = v0; v <= v1; ++v)
      acc = fma(p.alpha * p.B[j * p.ldb + (p.Bu + v - j)], p.A[v * p.lda + (p.Au + row - v)], acc);
    p.C[j * p.ldc + rc] = acc;
  }
}

// the columns outside the interior tiles [F0, F0 + ntiles*TJ) through the generic kernel
template <typename T>
static int gbmm_edges(GbmmParams<T> p, i64 F0, i64 F1, cudaStream_t stream, const char* name) {
  p.jskip0 = F0;
  p.jskip1 = F1;
  const i64 rest = (p.m - (F1 - F0)) * (i64)(p.Cl + p.Cu + 1);
  if (rest <= 0) return BM_OK;
  const i64 blocks = std::min<i64>(ceil_div(rest, 256), (i64)num_sms() * 32);
  gbmm_simple_kernel<T><<<(unsigned)blocks, 256, 0, stream>>>(p);
  return launch_status(name);
}

// Interior tiles through gbmm_reg_kernel and the remaining columns through the generic
// kernel.  Returns 1 (nothing launched) when the shapes do not qualify.
template <typename T, int M, int CPT>
static int gbmm_interior_launch(GbmmParams<T> p, RegTile rt, cudaStream_t stream, const char* name) {
  constexpr int TJ = kRegNT * CPT;
  const uint32_t nva = TJ + rt.NB - 1;
  const uint32_t a_el = CPT == 2 ? 2 * ((nva + 1) / 2) * rt.SA : nva * rt.SA;
  rt.ahalf = ((nva + 1) / 2) * rt.SA;
  rt.bhalf = (TJ / 2) * rt.SB;
  rt.chalf = (TJ / 2) * rt.SC;
  rt.boff = (a_el + 3) & ~3u;
  const size_t ab = ((size_t)rt.boff + (size_t)TJ * rt.SB) * sizeof(T);
  const size_t cb = (size_t)TJ * rt.SC * sizeof(T);
  const int smem = (int)std::max(ab, cb);
  const void* kfn = (const void*)gbmm_reg_kernel<T, M, M, CPT>;
  int r = cuda_status(ensure_smem(kfn, smem), name);
  if (r) return r;
  int per_sm = 0;
  r = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gbmm_reg_kernel<T, M, M, CPT>, kRegNT, smem),
                  name);
  if (r) return r;
  const i64 grid = std::min<i64>(rt.ntiles, (i64)num_sms() * std::max(per_sm, 1));
  gbmm_reg_kernel<T, M, M, CPT><<<(unsigned)grid, kRegNT, smem, stream>>>(p, rt);
  r = launch_status(name);
  if (r) return r;
  return gbmm_edges<T>(p, rt.F0, rt.F0 + rt.ntiles * TJ, stream, name);
}

template <int M>
static int gbmm_x2_launch(const GbmmParams<float>& p, X2Tile xt, cudaStream_t stream, const char* name) {
  const i64 nva = kX2TJ + xt.NB - 1;
  xt.a_elems = (uint32_t)((nva * p.lda + 4 + 3) & ~3ll);
  const i64 ab = (i64)xt.a_elems + kX2TJ * p.ldb + 4;
  const i64 cb = kX2TJ * p.ldc + 4;
  const int smem = 128 + (int)(std::max(ab, cb) * 4);
  if (smem > 227 * 1024) return 1;
  const void* kfn = (const void*)gbmm_f32x2_kernel<M, M>;
  int r = cuda_status(ensure_smem(kfn, smem), name);
  if (r) return r;
  int per_sm = 0;
  r = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gbmm_f32x2_kernel<M, M>, kX2NT, smem), name);
  if (r) return r;
  const i64 grid = std::min<i64>(xt.ntiles, (i64)num_sms() * std::max(per_sm, 1));
  gbmm_f32x2_kernel<M, M><<<(unsigned)grid, kX2NT, smem, stream>>>(p, xt);
  r = launch_status(name);
  if (r) return r;
  return gbmm_edges<float>(p, xt.F0, xt.F0 + xt.ntiles * kX2TJ, stream, name);
}

// Float32 with odd lda, ldc == Cl+Cu+1 and 16-byte aligned operands; 1 = not taken.
static int gbmm_interior_x2(const GbmmParams<float>& p, int cls, cudaStream_t stream, const char* name) {
  const int crows = p.Cl + p.Cu + 1;
  const bool aligned = ((reinterpret_cast<uintptr_t>(p.A) | reinterpret_cast<uintptr_t>(p.B) |
                         reinterpret_cast<uintptr_t>(p.C)) & 15) == 0;
  if (!aligned || (p.lda & 1) == 0 || p.ldc != crows || p.lda > 64 || p.ldb > 64) return 1;
  X2Tile xt;
  xt.NA = p.Al + p.Au + 1;
  xt.NB = p.Bl + p.Bu + 1;
  xt.NP = xt.NA + xt.NB - 1;
  xt.shift = p.Cu - (p.Au + p.Bu);
  // interior: every A, B term and every row of C's band inside the matrices; tiles start
  // at an even window column (j0 - Bu even)
  i64 F0 = std::max<i64>(p.Au + p.Bu, p.Cu);
  if ((F0 - p.Bu) & 1) ++F0;
  const i64 F1 = std::min(std::min(p.nu - p.Bl, p.n - p.Cl), p.m);
  xt.F0 = F0;
  xt.ntiles = F1 > F0 ? (F1 - F0) / kX2TJ : 0;
  if (xt.ntiles <= 0) return 1;
  xt.a_elems = 0;
  switch (cls) {
    case 9: return gbmm_x2_launch<9>(p, xt, stream, name);
    case 17: return gbmm_x2_launch<17>(p, xt, stream, name);
    default: return gbmm_x2_launch<33>(p, xt, stream, name);
  }
}

template <typename T>
static int gbmm_interior(const GbmmParams<T>& p, cudaStream_t stream, const char* name) {
  const int NA = p.Al + p.Au + 1, NB = p.Bl + p.Bu + 1;
  const int M = std::max(NA, NB);
  const int cls = M <= 9 ? 9 : M <= 17 ? 17 : M <= 33 ? 33 : 0;
  if (!cls || p.lda > 4096 || p.ldb > 4096 || p.ldc > 4096) return 1;
  if constexpr (sizeof(T) == 4) {
    const int r = gbmm_interior_x2(p, cls, stream, name);
    if (r != 1) return r;
  }
  constexpr int CPT = sizeof(T) == 4 ? 2 : 1;
  constexpr int TJ = kRegNT * CPT;
  RegTile rt;
  rt.NA = NA;
  rt.NB = NB;
  rt.rows_prod = NA + NB - 1;
  rt.shift = p.Cu - (p.Au + p.Bu);
  rt.SA = (uint32_t)(NA | 1);
  rt.SB = (uint32_t)(NB | 1);
  rt.SC = (uint32_t)(rt.rows_prod | 1);
  rt.F0 = p.Au + p.Bu;
  const i64 F1 = std::min(std::min(p.nu - p.Bl, p.n - p.Al - p.Bl), p.m);
  rt.ntiles = F1 > rt.F0 ? (F1 - rt.F0) / TJ : 0;
  if (rt.ntiles <= 0) return 1;
  rt.dlda = make_fastdiv((uint32_t)p.lda);
  rt.dldb = make_fastdiv((uint32_t)p.ldb);
  rt.dldc = make_fastdiv((uint32_t)p.ldc);
  switch (cls) {
    case 9: return gbmm_interior_launch<T, 9, CPT>(p, rt, stream, name);
    case 17: return gbmm_interior_launch<T, 17, CPT>(p, rt, stream, name);
    default: return gbmm_interior_launch<T, 33, CPT>(p, rt, stream, name);
  }
}

template <typename T>
static int gbmm_impl(i64 n, i64 nu, i64 m, i64 Al, i64 Au, i64 Bl, i64 Bu, i64 Cl, i64 Cu, T alpha, const T* A,
                     i64 lda, const T* B, i64 ldb, T beta, T* C, i64 ldc, cudaStream_t stream, const char* name) {
  if (n < 0) return -1;
  if (nu < 0) return -2;
  if (m < 0) return -3;
  if (Al < 0) return -4;
  if (Au < 0) return -5;
  if (Bl < 0) return -6;
  if (Bu < 0) return -7;
  // every in-matrix nonzero of A*B must fall inside C's band (bandwidths clipped to the
  // matrix size, as _bnds does, src/generic/broadcast.jl:895-897)
  if (Cl < std::min(Al + Bl, std::max<i64>(n - 1, 0))) return -8;
  if (Cu < std::min(Au + Bu, std::max<i64>(m - 1, 0))) return -9;
  if (lda < Al + Au + 1) return -12;
  if (ldb < Bl + Bu + 1) return -14;
  if (ldc < Cl + Cu + 1) return -17;
  if (n == 0 || m == 0) return BM_OK;
  if (Cl + Cu + 1 > (1 << 20) || Al + Au + 1 > (1 << 20)) return BM_ERR_UNSUPPORTED;

  GbmmParams<T> p;
  p.jskip0 = p.jskip1 = 0;
  p.n = n; p.nu = nu; p.m = m;
  p.Al = (int)Al; p.Au = (int)Au; p.Bl = (int)Bl; p.Bu = (int)Bu; p.Cl = (int)Cl; p.Cu = (int)Cu;
  p.lda = lda; p.ldb = ldb; p.ldc = ldc;
  p.alpha = alpha; p.beta = beta; p.A = A; p.B = B; p.C = C;
  p.status = status_word();
  const int nsm = num_sms();
  const i64 s = sizeof(T);
  const int crows = (int)(Cl + Cu + 1);
  const bool aligned =
      ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B) | reinterpret_cast<uintptr_t>(C)) & 15) == 0;

  // tile: TJ columns; a slot holds A (TJ+Bl+Bu cols), B (TJ cols), C (TJ cols if beta != 0)
  const i64 budget = 200 * 1024;
  const int stages = 2;
  const i64 slot = budget / stages - 512;
  const i64 per_col = (lda + ldb + (beta != T(0) ? ldc : 0)) * s;
  i64 tj = (slot - (Bl + Bu) * lda * s) / per_col;
  tj = std::min<i64>(tj, 512);
  const i64 want = ceil_div(m, (i64)nsm * 2);
  if (want < tj) tj = std::max<i64>(8, std::min<i64>(tj, want));
  const int kslots = (crows + 31) / 32;
  if (beta == T(0)) {
    const int r = gbmm_interior<T>(p, stream, name);
    if (r != 1) return r;  // 1: no interior tiles, fall through
  }
  if (!aligned || tj < 8 || kslots > 4) {
    const i64 total = m * (i64)crows;
    const int threads = 256;
    const i64 blocks = std::min<i64>(ceil_div(total, threads), (i64)nsm * 32);
    gbmm_simple_kernel<T><<<(unsigned)blocks, threads, 0, stream>>>(p);
    return launch_status(name);
  }
  p.tile = tj;
  p.ntiles = ceil_div(m, tj);
  p.stages = stages;
  const i64 q = 16 / s;
  const i64 abytes = (((tj + Bl + Bu) * lda + 2 * q) * s + 127) / 128 * 128;
  const i64 bbytes = ((tj * ldb + 2 * q) * s + 127) / 128 * 128;
  const i64 cbytes = beta != T(0) ? ((tj * ldc + 2 * q) * s + 127) / 128 * 128 : 0;
  p.boff = (uint32_t)abytes;
  p.coff = (uint32_t)(abytes + bbytes);
  p.stage_bytes = (uint32_t)(abytes + bbytes + cbytes);
  const int smem = 128 + stages * (int)p.stage_bytes;
  if (smem > 227 * 1024) {
    set_error("%s: tile selection exceeded shared memory (%d bytes)", name, smem);
    return BM_ERR_UNSUPPORTED;
  }
  const void* kfn = kslots == 1   ? (const void*)gbmm_tma_kernel<T, 1>
                    : kslots == 2 ? (const void*)gbmm_tma_kernel<T, 2>
                    : kslots == 3 ? (const void*)gbmm_tma_kernel<T, 3>
                                  : (const void*)gbmm_tma_kernel<T, 4>;
  int r = cuda_status(ensure_smem(kfn, smem), name);
  if (r) return r;
  const i64 grid = std::min<i64>(p.ntiles, nsm);
  switch (kslots) {
    case 1: gbmm_tma_kernel<T, 1><<<(unsigned)grid, 256, smem, stream>>>(p); break;
    case 2: gbmm_tma_kernel<T, 2><<<(unsigned)grid, 256, smem, stream>>>(p); break;
    case 3: gbmm_tma_kernel<T, 3><<<(unsigned)grid, 256, smem, stream>>>(p); break;
    default: gbmm_tma_kernel<T, 4><<<(unsigned)grid, 256, smem, stream>>>(p); break;
  }
  return launch_status(name);
}

// flags[r] = 1 when storage row r (one band) of an m x n band matrix holds a nonzero
// in-matrix entry (NaN counts as nonzero, as !iszero does).
template <typename T>
__global__ void band_nonzero_kernel(i64 m, i64 n, int l, int u, const T* __restrict__ A, i64 lda, int* flags) {
  const int rows = l + u + 1;
  const i64 total = n * (i64)rows;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
    const i64 j = e / rows;
    const int r = (int)(e - j * rows);
    const i64 k = j + r - u;
    if (k >= 0 && k < m && A[j * lda + r] != T(0)) flags[r] = 1;
  }
}

template <typename T>
static int nonzero_bands_impl(i64 m, i64 n, i64 l, i64 u, const T* A, i64 lda, int* flags, cudaStream_t stream,
                              const char* name) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (l + u + 1 < 0) return -4;
  if (lda < std::max<i64>(1, l + u + 1)) return -6;
  if (!flags) return -7;
  const i64 rows = l + u + 1;
  if (rows <= 0) return BM_OK;
  int r = cuda_status(cudaMemsetAsync(flags, 0, sizeof(int) * rows, stream), name);
  if (r || m == 0 || n == 0) return r;
  const i64 total = n * rows;
  const i64 blocks = std::min<i64>(ceil_div(total, 256), (i64)num_sms() * 16);
  band_nonzero_kernel<T><<<(unsigned)blocks, 256, 0, stream>>>(m, n, (int)l, (int)u, A, lda, flags);
  return launch_status(name);
}

}  // namespace bm

extern "C" int bm_dgb_nonzero_bands(int64_t m, int64_t n, int64_t l, int64_t u, const double* A, int64_t lda,
                                    int* flags, bm_stream_t stream) {
  return bm::nonzero_bands_impl<double>(m, n, l, u, A, lda, flags, reinterpret_cast<cudaStream_t>(stream),
                                        "bm_dgb_nonzero_bands");
}

extern "C" int bm_sgb_nonzero_bands(int64_t m, int64_t n, int64_t l, int64_t u, const float* A, int64_t lda,
                                    int* flags, bm_stream_t stream) {
  return bm::nonzero_bands_impl<float>(m, n, l, u, A, lda, flags, reinterpret_cast<cudaStream_t>(stream),
                                       "bm_sgb_nonzero_bands");
}

extern "C" int bm_dgbmm(int64_t n, int64_t nu, int64_t m, int64_t Al, int64_t Au, int64_t Bl, int64_t Bu, int64_t Cl,
                        int64_t Cu, double alpha, const double* A, int64_t lda, const double* B, int64_t ldb,
                        double beta, double* C, int64_t ldc, bm_stream_t stream) {
  return bm::gbmm_impl<double>(n, nu, m, Al, Au, Bl, Bu, Cl, Cu, alpha, A, lda, B, ldb, beta, C, ldc,
                               reinterpret_cast<cudaStream_t>(stream), "bm_dgbmm");
}

extern "C" int bm_sgbmm(int64_t n, int64_t nu, int64_t m, int64_t Al, int64_t Au, int64_t Bl, int64_t Bu, int64_t Cl,
                        int64_t Cu, float alpha, const float* A, int64_t lda, const float* B, int64_t ldb,
                        float beta, float* C, int64_t ldc, bm_stream_t stream) {
  return bm::gbmm_impl<float>(n, nu, m, Al, Au, Bl, Bu, Cl, Cu, alpha, A, lda, B, ldb, beta, C, ldc,
                              reinterpret_cast<cudaStream_t>(stream), "bm_sgbmm");
}
