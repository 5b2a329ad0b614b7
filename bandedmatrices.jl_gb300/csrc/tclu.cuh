// FP32 blocked banded LU with tensor-core trailing updates, for one wide-band system
// (64 <= kl + ku <= 256, kl <= 224): the factorization of the single-system refined
// solve (dsgbsv.cu).  No counterpart in the reference; per system it replaces the
// dgbtrf of lu! (src/banded/BandedLU.jl:98) when the caller refines the solution.
//
// One CTA of 8 warps on one SM.  With NB = 32 columns per panel, kvr = kl + ku and
// klr = kl both rounded up to multiples of 32, and R = klr + 32 window rows:
//
//   TMEM holds the trailing part of the active window, TRANSPOSED: a TMEM lane is a
//   band column and a TMEM column is a matrix row.  Column c lives in lane-ring
//   position c mod 256 (region (c mod 256) / 128 of the 512-column allocation, lane
//   c mod 128), row i in row-ring position i mod 256 of that region.  Warp w owns the
//   32 lanes of ring quarter w (region w / 4, lanes 32 (w % 4) ..): the only warp
//   allowed to touch them.  Invariant at the start of panel k (j0 = 32 k): TMEM holds
//   columns [j0, j0 + kvr) x rows [j0, j0 + klr), fully updated by panels < k.
//
//   Per panel:
//     1. wait for panel k-1's MMAs;
//     2. the panel quarter's warp copies its 32 columns (rows j0 .. j0+klr-1) from
//        TMEM to the shared-memory panel P; rows j0+klr .. j0+R-1 enter from the
//        staging buffer (FP64 band values rounded to FP32, loaded during the previous
//        panel): into P for the panel columns, into TMEM for the trailing quarters; the
//        columns j0+kvr .. j0+kvr+31 enter the free quarter, every window row (zero
//        outside the band);
//     3. partial-pivot LU of the R x 32 panel by the R/32 warps that hold a row each
//        (one named barrier among them per column): the pivot is the largest |a|
//        (exact to 2^-15 relative; the first row among near-equals); rows do not
//        move -- an interchange swaps the labels of the two window rows (it covers
//        the step's columns onward), the pivot row is read in place; scaling by the
//        rounded reciprocal, rank-1 update of the later panel columns; each column
//        goes to the FP32 factor storage as soon as it is final, at the rows of its
//        step (dgbtf2's layout, the one gbtrs reads); then every thread loads the
//        next panel's entering rows and columns from the FP64 band;
//     4. the panel's rows are put in their final order (every interchange applied,
//        dgetrf's order) for the update;
//     5. L21^T (R-32 rows x 32) is split into TF32 hi + lo (a = hi + lo, each rounded
//        to nearest) as the B operand;
//     6. each trailing quarter's warp applies the panel's interchanges to its TMEM
//        rows, solves U12 = L11^-1 A12 for its 32 columns (rows j0 .. j0+31, in
//        registers), stores U12 to the factor storage (column by column through the
//        warp's shared tile, so the stores coalesced) and writes it, split, as the A
//        operand (M = band columns, K = panel columns);
//     7. one thread issues, per TMEM region, D[cols, rows j0+32 ..] -= A B as three
//        kind::tf32 MMAs per K = 8 step (hi*hi + hi*lo + lo*hi: FP32-level products)
//        with the accumulator left in TMEM, and commits them to an mbarrier.
// Zero pivots are skipped (no interchange, scaling or update) and reported in info,
// as dgbtf2 does.  Every wait is bounded; on expiry the status word is set, the
// kernel stops, lets the issued MMAs finish (again bounded) and frees its TMEM.
#pragma once
#include "lu.cuh"
#include "tcgen05.cuh"

namespace bm {

constexpr int kTcNB = 32;
constexpr int kTcThreads = 256;

__host__ __device__ inline int tc_klr(int kl) { return ((kl + 31) / 32) * 32 < 32 ? 32 : ((kl + 31) / 32) * 32; }
__host__ __device__ inline int tc_kvr(int kl, int ku) { return ((kl + ku + 31) / 32) * 32; }
__host__ __device__ inline int tc_rs(int kl) { return tc_klr(kl) + kTcNB + 8; }  // == 8 (mod 32)

// Shared-memory layout (bytes).
constexpr int kTcHdr = 1024;
__host__ __device__ inline int tc_off_P() { return kTcHdr; }
__host__ __device__ inline int tc_off_A(int kl) { return kTcHdr + ((kTcNB * tc_rs(kl) * 4 + 1023) / 1024) * 1024; }
__host__ __device__ inline int tc_off_B(int kl) { return tc_off_A(kl) + 4 * 16384; }
__host__ __device__ inline int tc_off_T(int kl) { return tc_off_B(kl) + 2 * tc_klr(kl) * kTcNB * 4; }
// staging of the rows and columns the next panel brings in, FP32: [256 columns][32 rows]
// and [32 columns][64 rows], both XOR-swizzled on the row (conflict-free by row and by column)
__host__ __device__ inline int tc_off_S(int kl) { return tc_off_T(kl) + 8 * 32 * 32 * 4; }
__host__ __device__ inline int tc_smem_bytes(int kl) { return tc_off_S(kl) + (256 * 32 + 32 * 64) * 4; }

__host__ __device__ inline bool tc_lu_fits(long long kl, long long ku) {
  return kl >= 1 && ku >= 0 && kl + ku >= 64 && kl + ku <= 256 && kl <= 224;
}

// A: FP64 band ((kl+ku+1) x n, lda; A(i,c) at row ku + i - c), read only.
// F: FP32 gbtrf storage ((2kl+ku+1) x n, ldf; entry (i,c) at row kl + ku + i - c),
// written in full (fill-in rows included).  ipiv: n 1-based pivots.
__global__ void __launch_bounds__(kTcThreads, 1)
    sgbtrf_tc_kernel(i64 n, int kl, int ku, const double* __restrict__ A, i64 lda, float* __restrict__ F, i64 ldf,
                     i64* __restrict__ ipiv, i64* __restrict__ info, int* status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  if (!tc_lu_fits(kl, ku)) {  // the shared-memory layout and the TMEM ring assume these bounds
    if (threadIdx.x == 0) *info = -2;
    return;
  }
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int kv = kl + ku, klr = tc_klr(kl), kvr = tc_kvr(kl, ku), R = klr + kTcNB, RS = tc_rs(kl);
  const int nq = kvr / 32;  // trailing quarters per panel (1 .. 8)
  // ---- header
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem);
  int* abort_flag = reinterpret_cast<int*>(smem + 4);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 8);
  int* pivs = reinterpret_cast<int*>(smem + 64);              // [32] window-relative pivot rows
  uint32_t* wkey = reinterpret_cast<uint32_t*>(smem + 192);    // [2][8]
  uint8_t* slot_of = smem + 256;                              // [2][256]: slot of window row r
  float* P = reinterpret_cast<float*>(smem + tc_off_P());      // [32][RS]: panel column c, window row r
  float* Aop = reinterpret_cast<float*>(smem + tc_off_A(kl));  // region g: hi at 8192 g floats, lo 4096 after
  float* Bhi = reinterpret_cast<float*>(smem + tc_off_B(kl));  // [klr x 32] operand layout
  float* Blo = Bhi + klr * kTcNB;
  float* Tw = reinterpret_cast<float*>(smem + tc_off_T(kl)) + warp * 1024;  // [32 rows][32 lanes]
  float* Srow = reinterpret_cast<float*>(smem + tc_off_S(kl));  // new rows: column cr, row r at cr*32 + (r ^ (cr & 31))
  float* Scol = Srow + 256 * 32;                                 // new columns: q, row r at q*64 + (r ^ q)
  const int nw_lu = R / 32;  // warps of the panel factorization; the others stage the next panel

  // barrier of the panel-factorization warps only
  auto lu_sync = [&]() { asm volatile("bar.sync 1, %0;" ::"r"(32 * nw_lu) : "memory"); };
  auto aval = [&](i64 i, i64 c) -> float {
    const i64 d = i - c;
    return (i < n && c < n && d <= kl && d >= -ku) ? (float)A[(ku + d) + c * lda] : 0.0f;
  };
  if (warp == 0) tc::alloc(tslot, 512);
  if (tid == 0) {
    *abort_flag = 0;
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tbase = *tslot;
  // TMEM address of ring-row position rho in warp w's quarter
  auto taddr = [&](int w, int rho) -> uint32_t {
    return tbase + ((uint32_t)((w & 3) * 32) << 16) + (uint32_t)((w >> 2) * 256 + rho);
  };

  // ---- initial window: columns [0, kvr) x rows [0, klr)
  if (warp < nq) {
    const i64 c = 32 * warp + lane;
    for (int m = 0; m < klr / 32; ++m) {
      uint32_t v[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) v[i] = __float_as_uint(aval(32 * m + i, c));
      tc::st32(taddr(warp, 32 * m), v);
    }
    tc::wait_st();
  }
  // The rows and columns panel (j1 / 32) brings in, from the FP64 band, rounded to FP32:
  // rows j1+klr .. j1+klr+31 over its columns j1 .. j1+kvr-1 into Srow (warp w, lane r:
  // columns w, w+8, ..; 32 consecutive rows of a column per warp load), and the window's
  // last 64 rows over the 32 columns j1+kvr .. into Scol (zero outside the band and the
  // matrix).  Every thread issues its kStageRegs loads into registers, the panel
  // factorization runs while they are in flight, then they are rounded and stored.
  constexpr int kStageRegs = 40;
  double sv[kStageRegs];
  auto stage_issue = [&](i64 j1) {
    const double* Ab = A + j1 * lda;                 // column j1
    const int lim = (int)min(n - j1, (i64)1 << 30);  // rows / columns j1 + x exist for x < lim
#pragma unroll
    for (int q = 0; q < 32; ++q) {
      const int cc = warp + 8 * q, ri = klr + lane, d = ri - cc;
      sv[q] = (cc < kvr && ri < lim && cc < lim && d <= kl && d >= -ku) ? Ab[(ku + d) + (i64)cc * lda] : 0.0;
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int f = tid + kTcThreads * q, ri = klr - 32 + (f & 63), ci = kvr + (f >> 6), d = ri - ci;
      sv[32 + q] = (ri < lim && ci < lim && d <= kl && d >= -ku) ? Ab[(ku + d) + (i64)ci * lda] : 0.0;
    }
  };
  auto stage_store = [&]() {
#pragma unroll
    for (int q = 0; q < 32; ++q) {
      const int cc = warp + 8 * q;
      if (cc < kvr) Srow[cc * 32 + (lane ^ (cc & 31))] = (float)sv[q];
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int f = tid + kTcThreads * q;
      Scol[(f >> 6) * 64 + ((f & 63) ^ (f >> 6))] = (float)sv[32 + q];
    }
  };
  stage_issue(0);
  stage_store();
  __syncthreads();
  long long inf = 0;  // thread 0
  i64 k = 0;
  for (i64 j0 = 0; j0 < n; j0 += kTcNB, ++k) {
    const int jb = (int)min((i64)kTcNB, n - j0);
    const int wp = (int)(k & 7);
    // ---- 1. previous panel's MMAs
    if (k > 0) {
      if (tid == 0 && !mbar_wait(bar, (uint32_t)((k - 1) & 1))) {
        record_status(status, BM_STATUS_TIMEOUT);
        *abort_flag = 1;
      }
      __syncthreads();
      if (*abort_flag) break;
      tc::fence_after();
    }
    // ---- 2. panel out of TMEM; new rows and columns in
    if (warp == wp) {
      for (int m = 0; m < klr / 32; ++m) {
        uint32_t v[32];
        tc::ld32(taddr(wp, (int)((j0 + 32 * m) & 255)), v);
        tc::wait_ld();
        float* col = P + lane * RS + 32 * m;
#pragma unroll
        for (int q = 0; q < 8; ++q)
          *reinterpret_cast<float4*>(col + 4 * q) = make_float4(__uint_as_float(v[4 * q]), __uint_as_float(v[4 * q + 1]),
                                                               __uint_as_float(v[4 * q + 2]),
                                                               __uint_as_float(v[4 * q + 3]));
      }
    }
    for (int e = tid; e < 32 * 32; e += kTcThreads) {  // new rows, panel columns (staged)
      const int c = e >> 5, r = e & 31;
      P[c * RS + klr + r] = Srow[c * 32 + (r ^ c)];
    }
    {
      const int rel = (warp - wp + 8) & 7;
      const int relt = rel == 0 ? 8 : rel;  // position after the panel quarter: 1 .. 8
      if (relt == nq) {                     // new columns j0 + kvr + lane: every window row
        uint32_t v[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = 0u;  // rows above the band
        for (int m = 0; m < R / 32 - 2; ++m) tc::st32(taddr(warp, (int)((j0 + 32 * m) & 255)), v);
        for (int m = 0; m < 2; ++m) {
#pragma unroll
          for (int i = 0; i < 32; ++i) v[i] = __float_as_uint(Scol[lane * 64 + ((32 * m + i) ^ lane)]);
          tc::st32(taddr(warp, (int)((j0 + klr - 32 + 32 * m) & 255)), v);
        }
        tc::wait_st();
      } else if (relt < nq) {  // trailing quarter: the new rows (staged)
        const int cr = 32 * relt + lane;
        uint32_t v[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = __float_as_uint(Srow[cr * 32 + (i ^ lane)]);
        tc::st32(taddr(warp, (int)((j0 + klr) & 255)), v);
        tc::wait_st();
      }
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();

    // ---- 3. panel LU by the nw_lu warps, thread t holding slot t of the window (row t at
    // the panel's start).  Rows never move: an interchange swaps the window rows' labels
    // (lab: this slot's row; slot_of: the slot of a row, rewritten by every slot each
    // column), the pivot row is read in place, and each column's values go to the factor
    // storage as soon as they are final, at their row of that step -- dgbtf2's layout,
    // where an interchange covers the step's columns onward.  One named barrier per
    // column.  The pivot is the largest |a| (exact to 2^-15 relative), the first row
    // among near-equals.
    if (warp < nw_lu) {
      int lab = tid;
      bool moved = false;  // an interchange happened (warp-uniform)
      slot_of[tid] = (uint8_t)tid;
      lu_sync();
      float* Fcol = F + j0 * ldf + kv;  // row d of column j0 + c at Fcol[d] (advanced per column)
      for (int c = 0; c < jb; ++c) {
        const int par = c & 1;
        const float* Pc = P + c * RS;
        const bool cand = lab >= c && lab <= c + kl && j0 + lab < n;
        uint32_t key = 0u;
        if (cand) {
          uint32_t m = __float_as_uint(Pc[tid]) & 0x7fffffffu;
          m = m > 0x7f800000u ? 0u : m;  // NaN never wins
          key = (m & 0xffffff00u) | (uint32_t)(255 - lab);
        }
        key = __reduce_max_sync(0xffffffffu, key);
        if (lane == 0) wkey[par * 8 + warp] = key;
        lu_sync();
        const uint32_t best = __reduce_max_sync(0xffffffffu, lane < nw_lu ? wkey[par * 8 + lane] : 0u);
        const int p = 255 - (int)(best & 255u);  // the pivot row
        const int ps = slot_of[par * 256 + p];   // and its slot
        const float pv = Pc[ps];
        const bool nz = is_nonzero(pv);
        if (tid == 0) {
          ipiv[j0 + c] = j0 + p + 1;
          pivs[c] = nz ? p : c;
          if (!nz && inf == 0) inf = j0 + c + 1;
        }
        if (nz && p != c) {  // rows c and p trade places from this column on
          if (lab == c) lab = p;
          else if (lab == p) lab = c;
          moved = true;
        }
        slot_of[(par ^ 1) * 256 + lab] = (uint8_t)tid;
        float* Pt = P + tid;
        if (nz && lab > c && lab <= c + kl && j0 + lab < n) {
          // this row and the pivot row are different slots: declare it, so the loads of
          // the loop need not wait for its stores
          float* __restrict__ own = Pt;
          const float* __restrict__ piv = P + ps;
          const float l = own[c * RS] * __frcp_rn(pv);
          own[c * RS] = l;
#pragma unroll 4
          for (int c2 = c + 1; c2 < kTcNB; ++c2) own[c2 * RS] = fmaf(-l, piv[c2 * RS], own[c2 * RS]);
        }
        // column c is final in this slot: to the factor storage at this step's row
        const int d = lab - c;
        if (d <= kl && j0 + lab < n) Fcol[d] = Pt[c * RS];
        Fcol += ldf;
      }
      if (tid == 0)
        for (int c = jb; c < kTcNB; ++c) pivs[c] = c;
      if (moved) {  // the rows in their final order (every interchange applied), for the update
        float row[kTcNB];
#pragma unroll
        for (int c2 = 0; c2 < kTcNB; ++c2) row[c2] = P[c2 * RS + tid];
        lu_sync();
#pragma unroll
        for (int c2 = 0; c2 < kTcNB; ++c2) P[c2 * RS + lab] = row[c2];
      }
    }
    // the next panel's entering rows and columns, loaded after the factorization: loads in
    // flight during it saturated the SM's memory pipeline and slowed its shared-memory work
    stage_issue(j0 + kTcNB);
    stage_store();
    __syncthreads();
    // ---- 5. B operand: L21^T, rows r = 32 .. R-1 of the window (operand row r - 32)
    for (int e = tid; e < klr * kTcNB; e += kTcThreads) {
      // lanes cover one core matrix: 8 rows x 4 columns
      const int cm = e >> 5, w5 = e & 31;
      const int nn = (cm / 8) * 8 + (w5 & 7), c = (cm % 8) * 4 + (w5 >> 3);
      const float x = c < jb ? P[c * RS + kTcNB + nn] : 0.0f;
      const float h = tc::tf32_rna(x), lo = tc::tf32_rna(x - h);
      const uint32_t o = tc::op_off(nn, c, 8) >> 2;
      Bhi[o] = h;
      Blo[o] = lo;
    }
    // ---- 6. trailing quarters: interchanges, U12 = L11^-1 A12, U12 out, A operand
    {
      const int rel = (warp - wp + 8) & 7;
      const int relt = rel == 0 ? 8 : rel;
      float* Ah = Aop + (warp >> 2) * 8192;
      float* Al = Ah + 4096;
      const int mrow = (warp & 3) * 32 + lane;  // operand row in the region
      if (relt <= nq) {
        const i64 c = j0 + 32 * relt + lane;
        {
          uint32_t v[32];
          tc::ld32(taddr(warp, (int)(j0 & 255)), v);
          tc::wait_ld();
#pragma unroll
          for (int i = 0; i < 32; ++i) Tw[i * 32 + lane] = __uint_as_float(v[i]);
        }
        __syncwarp();
        for (int s = 0; s < jb; ++s) {
          const int p = pivs[s];
          if (p == s) continue;
          if (p < 32) {
            const float x = Tw[s * 32 + lane];
            Tw[s * 32 + lane] = Tw[p * 32 + lane];
            Tw[p * 32 + lane] = x;
          } else {
            const uint32_t ta = taddr(warp, (int)((j0 + p) & 255));
            const uint32_t x = tc::ld1(ta);
            tc::wait_ld();
            tc::st1(ta, __float_as_uint(Tw[s * 32 + lane]));
            tc::wait_st();
            Tw[s * 32 + lane] = __uint_as_float(x);
          }
        }
        float u[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) u[i] = Tw[i * 32 + lane];
#pragma unroll
        for (int kk = 0; kk < 32; ++kk) {
          const float* lk = P + kk * RS;
#pragma unroll
          for (int i = kk + 1; i < 32; ++i) u[i] = fmaf(-lk[i], u[kk], u[i]);
        }
        // U12 to the factor storage, a column per pass of the warp (lane = row)
        __syncwarp();
#pragma unroll
        for (int i = 0; i < 32; ++i) Tw[i * 32 + (lane ^ i)] = u[i];  // row i, column lane (swizzled)
        __syncwarp();
        for (int q = 0; q < 32; ++q) {
          const i64 cq = j0 + 32 * relt + q, d = (j0 + lane) - cq;  // U(j0+lane, cq): -kv <= d < 0
          if (cq < n && lane < jb && d >= -kv) F[(kv + d) + cq * ldf] = Tw[lane * 32 + (q ^ lane)];
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          float h[4], lo[4];
#pragma unroll
          for (int z = 0; z < 4; ++z) {
            h[z] = tc::tf32_rna(u[4 * q + z]);
            lo[z] = tc::tf32_rna(u[4 * q + z] - h[z]);
          }
          const uint32_t o = tc::op_off(mrow, 4 * q, 8) >> 2;
          *reinterpret_cast<float4*>(Ah + o) = make_float4(h[0], h[1], h[2], h[3]);
          *reinterpret_cast<float4*>(Al + o) = make_float4(lo[0], lo[1], lo[2], lo[3]);
        }
      } else {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const uint32_t o = tc::op_off(mrow, 4 * q, 8) >> 2;
          *reinterpret_cast<float4*>(Ah + o) = make_float4(0.f, 0.f, 0.f, 0.f);
          *reinterpret_cast<float4*>(Al + o) = make_float4(0.f, 0.f, 0.f, 0.f);
        }
      }
    }
    // ---- 7. A22 -= L21 U12 on the tensor cores, accumulator in TMEM
    fence_proxy_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (tid == 0) {
      const int rho0 = (int)((j0 + kTcNB) & 255);
      const int n1 = min(klr, 256 - rho0), n2 = klr - n1;
      const uint32_t bh = smem_u32(Bhi), bl = smem_u32(Blo);
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const uint32_t ah = smem_u32(Aop + g * 8192), al = ah + 16384;
        for (int piece = 0; piece < 2; ++piece) {
          const int N = piece ? n2 : n1;
          if (N <= 0) continue;
          const int rho = piece ? 0 : rho0, nstart = piece ? n1 : 0;
          const uint32_t d = tbase + (uint32_t)(g * 256 + rho);
          const uint32_t boff = (uint32_t)(nstart / 8) * 1024u;
          const uint32_t id = tc::idesc_tf32(128, N, true);
#pragma unroll
          for (int s = 0; s < kTcNB / 8; ++s) {
            const uint32_t ko = (uint32_t)s * 256u;
            const uint64_t dah = tc::sdesc(ah + ko, 128, 1024), dal = tc::sdesc(al + ko, 128, 1024);
            const uint64_t dbh = tc::sdesc(bh + boff + ko, 128, 1024), dbl = tc::sdesc(bl + boff + ko, 128, 1024);
            tc::mma_tf32(d, dah, dbh, id, 1u);
            tc::mma_tf32(d, dah, dbl, id, 1u);
            tc::mma_tf32(d, dal, dbh, id, 1u);
          }
        }
      }
      tc::commit(bar);
    }
  }
  // ---- the last MMAs, then free TMEM
  if (tid == 0 && k > 0) {
    if (!mbar_wait(bar, (uint32_t)((k - 1) & 1))) {
      record_status(status, BM_STATUS_TIMEOUT);
      (void)mbar_wait(bar, (uint32_t)((k - 1) & 1));
    }
    *info = inf;
  } else if (tid == 0) {
    *info = inf;
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (warp == 0) tc::dealloc(tbase, 512);
}

}  // namespace bm
