// FP32 factorization and solves of the mixed-precision refined solve (mixed.cu).
//
// The refined solve needs an FP32 LU with partial pivoting and its triangular
// solves, but not dgbtf2's exact operation order: accuracy is won back by the FP64
// refinement, and the result is fixed by the order below (deterministic, independent
// of the launch schedule).  So the FP32 factorization here is blocked, like LAPACK's
// dgbtrf, and both kernels are shaped for throughput across a batch:
//
// blk_lu_cta -- one CTA (kBlkThreads threads) per system.  The active part of the
//   matrix, rows j0 .. j0+NB+kl-1 and columns j0 .. j0+NB+kv-1 (kv = kl+ku), lives in
//   shared memory as a ring in both dimensions (row i in slot i mod RR, column c in
//   slot c mod CR), filled from the FP64 band and rounded on load.  Per panel of
//   NB = 16 columns:
//     1. warp 0 factors the panel in registers (one lane per row): partial pivot
//        (largest |a|, one warp reduction), interchange, scaling by the reciprocal
//        pivot, rank-1 update of the later panel columns; the interchanges are then
//        replayed on the earlier L columns, as dgetrf's panel leaves them;
//     2. every trailing column (one thread each) takes the panel's interchanges in
//        order and the triangular solve U12 = L11^-1 A12 (16 rows, in registers);
//     3. A22 -= L21 U12 by 4x4 register tiles (float4 shared-memory loads of L21);
//     4. the panel columns (written before the replay: band storage keeps column k's
//        multipliers as step k left them, the layout gbtrs reads) and the U12 rows go
//        to the FP32 factor storage;
//     5. the window slides by 16 rows and columns; the elements it brings in are
//        copied from the FP64 band with cp.async while steps 1-4 run (or, when the
//        staging buffer would cost an SM a CTA, loaded at the slide).
//   Zero pivots are skipped (no interchange, no scaling, no update) and reported in
//   info, as dgbtf2 does.
//
// blk_solve_warp -- one warp solves up to 4 right-hand sides of a system: lane l
//   keeps rows i = l (mod 32) of the window in registers (a ring of NS slots per
//   right-hand side).  Forward sweep (dgbtrs 'N'): interchange b(j) with
//   b(ipiv(j)) by two shuffles, then b(j+1 .. j+kl) -= L(:, j) b(j), one fma per lane
//   and slot.  Back substitution (U, bandwidth kv): x(j) = b(j) * (1 / U(j,j)), then
//   b(j-kv .. j-1) -= U(:, j) x(j).  The step's L or U column is read from the factor
//   storage into a shared-memory ring 8 steps ahead (cp.async; prefetched to L2 32
//   steps ahead), and the rows entering the window and the pivots are loaded one
//   32-step chunk ahead.
#pragma once
#include "lu.cuh"

namespace bm {

constexpr int kBlkNB = 16;
constexpr int kBlkThreads = 128;

__host__ __device__ inline int blk_rr(int kl) { return (kBlkNB + kl + 3) / 4 * 4; }
// column stride: a multiple of 4 (float4 rows) that is 4 mod 8 (4-way bank spread for
// accesses along a row)
__host__ __device__ inline int blk_rs(int kl) {
  const int rr = blk_rr(kl);
  return rr % 8 == 4 ? rr : rr + 4;
}
__host__ __device__ inline int blk_cr(int kl, int ku) { return kBlkNB + kl + ku; }
constexpr int kBlkHdrBytes = 128;
// header, the FP32 window, and the FP64 staging of the elements the next slide brings
// in (16 new rows over C columns, 16 new columns over kl rows)
__host__ __device__ inline i64 blk_smem_bytes(i64 kl, i64 ku, bool stage = true) {
  return kBlkHdrBytes + (i64)blk_rs((int)kl) * blk_cr((int)kl, (int)ku) * 4 +
         (stage ? ((i64)blk_cr((int)kl, (int)ku) * kBlkNB + (i64)kBlkNB * kl) * 8 : 0);
}

// Factors system (n, kl, ku) from the FP64 band A (gbtrf storage: A(i,c) at row
// kv + i - c, the matrix in rows kl..) into the FP32 storage A32 (same layout) and
// ipiv (1-based).  Called by all kBlkThreads threads; returns info in every thread.
static __device__ i64 blk_lu_cta(i64 n, int kl, int ku, const double* __restrict__ A, i64 ldab, float* __restrict__ A32,
                          i64 ldab32, i64* __restrict__ ipiv, unsigned char* smem, bool stage) {
  constexpr int NB = kBlkNB, NT = kBlkThreads;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int kv = kl + ku, R = NB + kl, RR = blk_rr(kl), RS = blk_rs(kl), C = NB + kv, CR = C;
  int* piv = reinterpret_cast<int*>(smem);  // [NB] panel pivot offsets (-1: zero pivot)
  long long* sinfo = reinterpret_cast<long long*>(smem + 64);
  float* W = reinterpret_cast<float*>(smem + kBlkHdrBytes);
  double* SR = reinterpret_cast<double*>(W + (i64)RS * CR);  // [C][NB]: new rows, by column
  double* SC = SR + (i64)C * NB;                             // [NB][kl]: new columns
  auto inband = [&](i64 i, i64 c) {
    const i64 d = i - c;
    return i >= 0 && c >= 0 && i < n && c < n && d <= kl && d >= -ku;
  };
  // the next slide's elements (original values, untouched by the factorization so
  // far) are copied with cp.async while the current panel is factored
  auto stage_slide = [&](i64 nj) {
    for (int e = tid; e < NB * C; e += NT) {
      const int c = e >> 4, rr = e & (NB - 1);  // new-frame column c, new row kl + rr
      const i64 i = nj + kl + rr, col = nj + c;
      const bool ok = inband(i, col);
      cp_async_elem(SR + e, ok ? A + (kv + i - col) + col * ldab : A, ok);
    }
    for (int e = tid; e < NB * kl; e += NT) {
      const int cc = e / kl, r = e - cc * kl;  // new-frame column C-NB+cc, row r
      const i64 i = nj + r, col = nj + C - NB + cc;
      const bool ok = inband(i, col);
      cp_async_elem(SC + e, ok ? A + (kv + i - col) + col * ldab : A, ok);
    }
    cp_async_commit();
  };
  int rb = 0, cb = 0;  // slots of row j0 and column j0
  // slot of window row r / column c: rb + r < 3 RR and cb + c < 3 CR hold for every
  // argument below (r < RR + NB, c < CR + NB, RR and CR >= NB)
  auto rs = [&](int r) {
    int t = rb + r;
    t = t >= RR ? t - RR : t;
    return t >= RR ? t - RR : t;
  };
  auto cs = [&](int c) {
    int t = cb + c;
    t = t >= CR ? t - CR : t;
    return t >= CR ? t - CR : t;
  };
  if (n <= 0) return 0;
  // initial window, eight loads in flight per thread
  for (int e0 = 0; e0 < R * C; e0 += 8 * NT) {
    float v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int e = e0 + k * NT + tid;
      const int c = e / R, r = e - c * R;
      double a = 0.0;
      if (e < R * C && inband(r, c)) a = A[(kv + r - c) + (i64)c * ldab];
      v[k] = (float)a;
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int e = e0 + k * NT + tid;
      const int c = e / R, r = e - c * R;
      if (e < R * C) W[c * RS + r] = v[k];
    }
  }
  if (tid == 0) *sinfo = 0;
  __syncthreads();
  for (i64 j0 = 0; j0 < n; j0 += NB) {
    const int jb = (int)min((i64)NB, n - j0);
    if (stage && j0 + jb < n) stage_slide(j0 + NB);
    // ---- 1. panel, by warp 0, in registers: lane L holds window rows L + 32k (k < 3)
    // of the panel's NB columns.  Step cc swaps rows cc and its pivot row in columns
    // cc.. only, so the L columns leave the panel as dgbtf2 leaves them (band storage
    // order, written back below); the interchanges of later steps are replayed on the
    // L columns in shared memory afterwards for the trailing update.
    if (warp == 0) {
      long long info = *sinfo;
      float w[3][NB];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int r = lane + 32 * k;
#pragma unroll
        for (int c = 0; c < NB; ++c) w[k][c] = r < R ? W[cs(c) * RS + rs(r)] : 0.0f;
      }
#pragma unroll
      for (int cc = 0; cc < NB; ++cc) {
        if (cc < jb) {
          const i64 j = j0 + cc;
          const int km = (int)min((i64)kl, n - 1 - j);
          bool inr[3];  // rows cc+1 .. cc+km (the multipliers' rows)
          // Partial pivoting by one warp reduction: the key is |a| with its 7 low bits
          // replaced by 127 - row, so the largest magnitude wins and, among magnitudes
          // equal to 2^-16 relative, the first row (a stable pivot; the refinement
          // does not need idamax's exact choice).  NaN keys never win.
          unsigned key = 0u;
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const int r = lane + 32 * k;
            inr[k] = r > cc && r <= cc + km;
            if (r >= cc && r <= cc + km) {
              unsigned m = __float_as_uint(w[k][cc]) & 0x7fffffffu;
              m = m > 0x7f800000u ? 0u : m;
              key = max(key, (m & 0xffffff80u) | (unsigned)(127 - r));
            }
          }
          const int p = 127 - (int)(__reduce_max_sync(0xffffffffu, key) & 127u);  // pivot row (window index)
          const int pk = p >> 5, pl = p & 31;
          auto slot = [&](int c) { return pk == 0 ? w[0][c] : pk == 1 ? w[1][c] : w[2][c]; };
          const float pv = __shfl_sync(0xffffffffu, slot(cc), pl);
          const bool nz = is_nonzero(pv);
          if (lane == 0) {
            piv[cc] = nz ? p - cc : -1;
            ipiv[j] = j + (p - cc) + 1;
          }
          if (nz) {
            float u[NB];
            if (p != cc) {
#pragma unroll
              for (int c = cc; c < NB; ++c) {
                const float a = __shfl_sync(0xffffffffu, w[0][c], cc);  // row cc (lane cc, slot 0)
                const float b = __shfl_sync(0xffffffffu, slot(c), pl);  // the pivot row
                if (lane == cc) w[0][c] = b;
                if (lane == pl) {
                  if (pk == 0) w[0][c] = a;
                  else if (pk == 1) w[1][c] = a;
                  else w[2][c] = a;
                }
                u[c] = b;
              }
            } else {  // no interchange: broadcast row cc
#pragma unroll
              for (int c = cc + 1; c < NB; ++c) u[c] = __shfl_sync(0xffffffffu, w[0][c], cc);
            }
            const float rcp = __frcp_rn(pv);
#pragma unroll
            for (int k = 0; k < 3; ++k)
              if (inr[k]) w[k][cc] *= rcp;
#pragma unroll
            for (int c = cc + 1; c < NB; ++c)
#pragma unroll
              for (int k = 0; k < 3; ++k)
                if (inr[k]) w[k][c] = fmaf(-w[k][cc], u[c], w[k][c]);
          } else if (info == 0) {
            info = j + 1;
          }
        }
      }
      // the panel's columns, as dgbtf2 leaves them: to the window and to the factor storage
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int r = lane + 32 * k;
#pragma unroll
        for (int c = 0; c < NB; ++c)
          if (c < jb && r < R) {
            W[cs(c) * RS + rs(r)] = w[k][c];
            if (r >= c - kv && r <= c + kl && j0 + r < n) A32[(kv + r - c) + (j0 + c) * ldab32] = w[k][c];
          }
      }
      if (lane == 0) *sinfo = info;
    }
    __syncthreads();
    // the later steps' interchanges on the panel's L columns (dgetrf's order), which the
    // triangular solve and the trailing update use
    if (tid < jb) {
      float* cl = W + cs(tid) * RS;
      for (int cc = tid + 1; cc < jb; ++cc) {
        const int p = piv[cc];
        if (p > 0) {
          const int a = rs(cc), b = rs(cc + p);
          const float x = cl[a];
          cl[a] = cl[b];
          cl[b] = x;
        }
      }
    }
    __syncthreads();
    // ---- 2. trailing columns: interchanges in order, then U12 = L11^-1 A12
    const int ntc = (int)min((i64)(C - jb), n - (j0 + jb));
    for (int t = tid; t < ntc; t += NT) {
      float* cl = W + cs(jb + t) * RS;
      for (int cc = 0; cc < jb; ++cc) {
        const int p = piv[cc];
        if (p > 0) {
          const int a = rs(cc), b = rs(cc + p);
          const float x = cl[a];
          cl[a] = cl[b];
          cl[b] = x;
        }
      }
      float u[NB];
#pragma unroll
      for (int k = 0; k < NB; ++k) u[k] = k < jb ? cl[rs(k)] : 0.0f;
#pragma unroll
      for (int k = 0; k < NB; ++k) {
        const float* lk = W + cs(k) * RS;
#pragma unroll
        for (int i = k + 1; i < NB; ++i) u[i] = fmaf(-lk[rs(i)], u[k], u[i]);
      }
#pragma unroll
      for (int k = 0; k < NB; ++k)
        if (k < jb) cl[rs(k)] = u[k];
    }
    __syncthreads();
    // ---- 3. A22 -= L21 U12: rows jb .. jb+kl-1, trailing columns, 4x4 tiles
    if (ntc > 0) {
      const int nrg = (kl + 3) >> 2, ncg = (ntc + 3) >> 2;
      for (int t = tid; t < nrg * ncg; t += NT) {
        const int cg = t / nrg, rg = t - cg * nrg;
        const int r0 = rs(jb + 4 * rg);  // 4-aligned, no wrap inside the group
        float* cp[4];
        bool cv[4];
        float4 acc[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int c = 4 * cg + q;
          cv[q] = c < ntc;
          cp[q] = W + cs(jb + (cv[q] ? c : 0)) * RS;
          acc[q] = cv[q] ? *reinterpret_cast<const float4*>(cp[q] + r0) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        for (int k = 0; k < jb; ++k) {
          const float4 l = *reinterpret_cast<const float4*>(W + cs(k) * RS + r0);
          const int qk = rs(k);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const float u = -cp[q][qk];
            acc[q].x = fmaf(l.x, u, acc[q].x);
            acc[q].y = fmaf(l.y, u, acc[q].y);
            acc[q].z = fmaf(l.z, u, acc[q].z);
            acc[q].w = fmaf(l.w, u, acc[q].w);
          }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (cv[q]) *reinterpret_cast<float4*>(cp[q] + r0) = acc[q];
      }
    }
    __syncthreads();
    // ---- 4. U12 rows to the factor storage (the panel columns went out in step 1)
    {
      // U12: rows 0 .. jb-1 of the trailing columns
      for (int e = tid; e < ntc * NB; e += NT) {
        const int t = e / NB, r = e - t * NB;
        const int c = jb + t;
        if (r < jb && c - r <= kv) A32[(kv + r - c) + (j0 + c) * ldab32] = W[cs(c) * RS + rs(r)];
      }
    }
    if (j0 + jb >= n) break;
    __syncthreads();
    // ---- 5. slide by NB: new rows (old-frame R .. R+NB-1) over the new frame's columns,
    // new columns (old-frame C .. C+NB-1) over the retained rows
    if (stage) {
      cp_async_wait<0>();
      __syncthreads();
      for (int e = tid; e < NB * C; e += NT) {
        const int c = e >> 4, rr = e & (NB - 1);  // new-frame column c, new row kl + rr
        W[cs(NB + c) * RS + rs(R + rr)] = (float)SR[e];
      }
      for (int e = tid; e < NB * kl; e += NT) {
        const int cc = e / kl, r = e - cc * kl;  // new-frame column C-NB+cc, row r
        W[cs(C + cc) * RS + rs(NB + r)] = (float)SC[e];
      }
    } else {  // no staging buffer (more CTAs per SM): eight loads in flight per thread
      const i64 nj = j0 + NB;
      const int n1 = NB * C, tot = n1 + NB * kl;
      for (int e0 = 0; e0 < tot; e0 += 8 * NT) {
        float v[8];
        int slot[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int e = e0 + q * NT + tid;
          double a = 0.0;
          slot[q] = -1;
          if (e < tot) {
            i64 i, col;
            if (e < n1) {
              const int c = e >> 4, rr = e & (NB - 1);
              i = nj + kl + rr;
              col = nj + c;
              slot[q] = cs(NB + c) * RS + rs(R + rr);
            } else {
              const int f = e - n1, cc = f / kl, r = f - cc * kl;
              i = nj + r;
              col = nj + C - NB + cc;
              slot[q] = cs(C + cc) * RS + rs(NB + r);
            }
            if (inband(i, col)) a = A[(kv + i - col) + col * ldab];
          }
          v[q] = (float)a;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (slot[q] >= 0) W[slot[q]] = v[q];
      }
    }
    __syncthreads();
    rb = rs(NB);
    cb = cs(NB);
  }
  __syncthreads();
  const i64 info = *sinfo;
  __syncthreads();
  return info;
}

// ---------------------------------------------------------------- warp solves
// Value of slot s (runtime) among NS registers.
template <int NS>
__device__ __forceinline__ float slot_get(const float (&v)[NS], int s) {
  float r = v[0];
#pragma unroll
  for (int k = 1; k < NS; ++k) r = s == k ? v[k] : r;
  return r;
}
template <int NS>
__device__ __forceinline__ void slot_set(float (&v)[NS], int s, float x, bool doit) {
#pragma unroll
  for (int k = 0; k < NS; ++k) v[k] = (doit && s == k) ? x : v[k];
}

// Each step's L or U column is copied kSolveD steps ahead (cp.async, one group per
// step) into a per-warp shared-memory ring of kSolveD + 1 entries, each lane copying
// the entries of its own rows, so no warp synchronisation is needed; columns are also
// prefetched to L2 kSolvePF steps ahead.  The copies for step j + kSolveD are made
// with the rows the lane holds at step j: a slot that changes hands before then held
// a row that has left the window (zero multiplier, which is right), and its new row
// lies beyond that step's band when the window holds W >= band + 1 + kSolveD rows.
constexpr int kSolveD = 8;
constexpr int kSolvePF = 32;
constexpr int kSolveNR = 4;  // right-hand sides per sweep
__host__ __device__ constexpr int blk_ns(int band) { return (band + 1 + kSolveD + 31) / 32; }
// ring floats per warp: (kSolveD + 1) entries of 5 slots x 32 lanes + the diagonal x 32
constexpr int kSolveRingStride = 6 * 32;
constexpr int kSolveRingFloats = (kSolveD + 1) * kSolveRingStride;

// Forward sweep (dgbtrs 'N': interchange, then b(j+1:j+lm) -= b(j) L(j+1:j+lm, j)) for
// nr <= NR right-hand sides B[:, 0..nr) (leading dim ldb); 32*NS >= kl+1+kSolveD.  The
// ring holds kSolveD + 1 entries of STRIDE floats (STRIDE >= 32*NS).
template <int NS, int NR = kSolveNR, int STRIDE = kSolveRingStride>
__device__ __noinline__ void blk_fwd_warp(i64 n, int kl, int ku, int nr, const float* __restrict__ A32, i64 ldab,
                                          const i64* __restrict__ ipiv, float* __restrict__ B, i64 ldb,
                                          float* ring, int lane) {
  constexpr int W = 32 * NS, D = kSolveD;
  static_assert(STRIDE >= 32 * NS, "ring entry too small");
  if (kl == 0 || n <= 1) return;
  const int kv = kl + ku;
  const i64 nst = n - 1;  // steps j = 0 .. n-2
  float b[NR][NS];
  i64 row[NS];
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    row[s] = lane + 32 * s;
#pragma unroll
    for (int c = 0; c < NR; ++c) {
      float v = 0.0f;
      if (c < nr && row[s] < n) v = B[row[s] + c * ldb];
      b[c][s] = v;
    }
  }
  // copies of step j's multipliers into ring entry e (rows held now)
  auto issue = [&](i64 j, int e) {
    const int lm = j < nst ? (int)min((i64)kl, n - 1 - j) : 0;
    float* dst = ring + e * STRIDE + lane;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      const i64 d = row[s] - j;
      const bool ok = d >= 1 && d <= lm;
      cp_async_elem(dst + 32 * s, ok ? A32 + (kv + d) + j * ldab : A32, ok);
    }
    cp_async_commit();
  };
  for (int u = 0; u < D; ++u) issue(u, u);
  float ent[NR];
  auto load_ent = [&](i64 j0c) {  // rows j + W for the chunk's steps j, lane j mod 32
    const i64 r = j0c + W + lane;
#pragma unroll
    for (int c = 0; c < NR; ++c) {
      float v = 0.0f;
      if (c < nr && r < n) v = B[r + c * ldb];
      ent[c] = v;
    }
  };
  load_ent(0);
  i64 pv_next = lane < nst ? ipiv[lane] - 1 : 0;
  int er = 0, ew = D;  // ring entries read at this step and refilled for step j + D
  for (i64 j0 = 0; j0 < nst; j0 += 32) {
    float cur[NR];
#pragma unroll
    for (int c = 0; c < NR; ++c) cur[c] = ent[c];
    if (j0 + 32 < nst) load_ent(j0 + 32);
    const i64 pv_lane = pv_next;  // the chunk's pivots, one per lane
    pv_next = j0 + 32 + lane < nst ? ipiv[j0 + 32 + lane] - 1 : 0;
    const int cn = (int)min((i64)32, nst - j0);
    for (int t = 0; t < cn; ++t) {
      const i64 j = j0 + t;
      if (lane < max(3, (kl + 31) / 32) && j + kSolvePF < nst) {
        const float* pf = A32 + (kv + 1) + (j + kSolvePF) * ldab + min(lane * 32, kl - 1);
        asm volatile("prefetch.global.L2 [%0];" ::"l"(pf));
      }
      cp_async_wait<D - 1>();
      float l[NS];
#pragma unroll
      for (int s = 0; s < NS; ++s) l[s] = ring[er * STRIDE + 32 * s + lane];
      issue(j + D, ew);
      er = er == D ? 0 : er + 1;
      ew = ew == D ? 0 : ew + 1;
      const i64 p = __shfl_sync(0xffffffffu, pv_lane, t);
      const int sj = (int)((j >> 5) % NS), lp = (int)(p & 31), sp = (int)((p >> 5) % NS);
#pragma unroll
      for (int c = 0; c < NR; ++c) {
        const float vj = __shfl_sync(0xffffffffu, slot_get<NS>(b[c], sj), t);
        const float vp = __shfl_sync(0xffffffffu, slot_get<NS>(b[c], sp), lp);
        const float x = vp;  // b(j) after the interchange (vp == vj when p == j)
        slot_set<NS>(b[c], sp, vj, lane == lp && p != j);
        if (lane == t && c < nr) B[j + c * ldb] = x;
#pragma unroll
        for (int s = 0; s < NS; ++s) b[c][s] = fmaf(-l[s], x, b[c][s]);
      }
      // row j leaves lane t's slot sj; row j + W enters it
      if (lane == t) {
        row[sj] = j + W;
#pragma unroll
        for (int c = 0; c < NR; ++c) slot_set<NS>(b[c], sj, cur[c], true);
      }
    }
  }
  cp_async_wait<0>();
  // the last row: b(n-1) is final
  {
    const i64 j = n - 1;
    const int sj = (int)((j >> 5) % NS);
#pragma unroll
    for (int c = 0; c < NR; ++c) {
      const float v = slot_get<NS>(b[c], sj);
      if (lane == (int)(j & 31) && c < nr) B[j + c * ldb] = v;
    }
  }
  __syncwarp();
}

// Back substitution with U (bandwidth kv, dtbsv 'U','N'): x(j) = b(j) * (1/U(j,j)),
// then b(j-kv .. j-1) -= x(j) U(:, j); 32*NS >= kv + 1 + kSolveD.  Ring entries of
// STRIDE floats hold NS slots and, in the last 32 floats, the diagonal.
template <int NS, int NR = kSolveNR, int STRIDE = kSolveRingStride>
__device__ __noinline__ void blk_bwd_warp(i64 n, int kv, int nr, const float* __restrict__ A32, i64 ldab,
                                          float* __restrict__ B, i64 ldb, float* ring, int lane) {
  constexpr int W = 32 * NS, D = kSolveD, DG = STRIDE / 32 - 1;
  static_assert(STRIDE >= 32 * (NS + 1), "ring entry too small");
  if (n <= 0) return;
  float b[NR][NS];
  i64 row[NS];
  // lane l, slot s holds the row i = l (mod 32) with (i >> 5) mod NS == s in (j - W, j]
  const i64 top = n - 1;
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    // rows top - W + 1 .. top: i0 is the last one held by this lane, in slot
    // (i0 >> 5) mod NS; the row in slot s is k = ((i0 >> 5) - s) mod NS rows of 32 below
    const i64 i0 = top - ((top - lane) & 31);
    const i64 k = (((i0 >> 5) - s) % NS + NS) % NS;
    const i64 r = i0 - 32 * k;
    row[s] = r;
#pragma unroll
    for (int c = 0; c < NR; ++c) {
      float v = 0.0f;
      if (c < nr && r >= 0) v = B[r + c * ldb];
      b[c][s] = v;
    }
  }
  auto issue = [&](i64 j, int e) {  // step j's U column (and diagonal) into ring entry e
    float* dst = ring + e * STRIDE + lane;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      const i64 d = j - row[s];
      const bool ok = j >= 0 && d >= 1 && d <= kv && row[s] >= 0;
      cp_async_elem(dst + 32 * s, ok ? A32 + (kv - d) + j * ldab : A32, ok);
    }
    cp_async_elem(dst + 32 * DG, j >= 0 ? A32 + kv + j * ldab : A32, j >= 0);
    cp_async_commit();
  };
  for (int u = 0; u < D; ++u) issue(top - u, u);
  float ent[NR];
  auto load_ent = [&](i64 j0c) {  // rows j - W for the chunk's steps j = j0c, j0c-1, ..: lane = j mod 32
    const i64 jj = j0c - ((j0c - lane) & 31);  // the chunk's step held by this lane
    const i64 r = jj - W;
#pragma unroll
    for (int c = 0; c < NR; ++c) {
      float v = 0.0f;
      if (c < nr && r >= 0) v = B[r + c * ldb];
      ent[c] = v;
    }
  };
  load_ent(top);
  int er = 0, ew = D;
  for (i64 j0 = top; j0 >= 0; j0 -= 32) {
    float cur[NR];
#pragma unroll
    for (int c = 0; c < NR; ++c) cur[c] = ent[c];
    if (j0 - 32 >= 0) load_ent(j0 - 32);
    const int cn = (int)min((i64)32, j0 + 1);
    for (int t = 0; t < cn; ++t) {
      const i64 j = j0 - t;
      if (lane < max(5, (kv + 32) / 32) && j - kSolvePF >= 0) {
        const float* pf = A32 + (j - kSolvePF) * ldab + min(lane * 32, kv);
        asm volatile("prefetch.global.L2 [%0];" ::"l"(pf));
      }
      cp_async_wait<D - 1>();
      float uc[NS];
      const float* src = ring + er * STRIDE + lane;
#pragma unroll
      for (int s = 0; s < NS; ++s) uc[s] = src[32 * s];
      const float rcp = __frcp_rn(src[32 * DG]);
      issue(j - D, ew);
      er = er == D ? 0 : er + 1;
      ew = ew == D ? 0 : ew + 1;
      const int lj = (int)(j & 31), sj = (int)((j >> 5) % NS);
#pragma unroll
      for (int c = 0; c < NR; ++c) {
        const float x = __shfl_sync(0xffffffffu, slot_get<NS>(b[c], sj), lj) * rcp;
        if (lane == lj && c < nr) B[j + c * ldb] = x;
#pragma unroll
        for (int s = 0; s < NS; ++s) b[c][s] = fmaf(-uc[s], x, b[c][s]);
      }
      if (lane == lj) {
        row[sj] = j - W;
#pragma unroll
        for (int c = 0; c < NR; ++c) slot_set<NS>(b[c], sj, cur[c], true);
      }
    }
  }
  cp_async_wait<0>();
  __syncwarp();
}

// gbtrs 'N' with the FP32 factors for right-hand sides [c0, c0+nr) of B (nr <=
// kSolveNR), by one warp; ring: kSolveRingFloats of this warp's shared memory.
static __device__ void blk_solve_warp(i64 n, int kl, int ku, int nr, const float* A32, i64 ldab, const i64* ipiv, float* B,
                               i64 ldb, float* ring, int lane) {
  const int kv = kl + ku;
  switch (blk_ns(kl)) {
    case 1: blk_fwd_warp<1>(n, kl, ku, nr, A32, ldab, ipiv, B, ldb, ring, lane); break;
    case 2: blk_fwd_warp<2>(n, kl, ku, nr, A32, ldab, ipiv, B, ldb, ring, lane); break;
    default: blk_fwd_warp<3>(n, kl, ku, nr, A32, ldab, ipiv, B, ldb, ring, lane); break;
  }
  switch (blk_ns(kv)) {
    case 1: blk_bwd_warp<1>(n, kv, nr, A32, ldab, B, ldb, ring, lane); break;
    case 2: blk_bwd_warp<2>(n, kv, nr, A32, ldab, B, ldb, ring, lane); break;
    case 3: blk_bwd_warp<3>(n, kv, nr, A32, ldab, B, ldb, ring, lane); break;
    case 4: blk_bwd_warp<4>(n, kv, nr, A32, ldab, B, ldb, ring, lane); break;
    default: blk_bwd_warp<5>(n, kv, nr, A32, ldab, B, ldb, ring, lane); break;
  }
}
// the blocked LU holds the panel's rows in three register slots (NB + kl <= 96), the
// solves their windows in at most 3 (forward) and 5 (backward) slots
__host__ __device__ inline bool blk_lu_fits(i64 kl, i64 ku) { return kl >= 0 && ku >= 0 && kl <= 96 - kBlkNB; }
__host__ __device__ inline bool blk_solve_fits(i64 kl, i64 ku) {
  return kl >= 0 && ku >= 0 && blk_ns((int)kl) <= 3 && blk_ns((int)(kl + ku)) <= 5;
}

}  // namespace bm
