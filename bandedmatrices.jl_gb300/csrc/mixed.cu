// Mixed-precision refined banded solves (no counterpart in the reference; an
// addition beside lu!/ldiv!, src/banded/BandedLU.jl:90-103,
// src/banded/linalg.jl:24-30).
//
// Per system s the FP64 band A is rounded to an FP32 copy in gbtrf storage and
// factored in FP32 with partial pivoting (the group algorithms of lu.cuh /
// lureg.cuh).  Then, for its right-hand sides B,
//     X = FP64(LU32 \ FP32(B))
//     repeat: R = B - A X                    (FP64, from the original FP64 band)
//             berr = max_c ||r_c||_inf / (||A||_inf ||x_c||_inf + ||b_c||_inf)
//             stop when berr <= tol or after maxit corrections
//             X = X + FP64(LU32 \ FP32(R))
// The residual and the update, the steps whose stability needs it, run in FP64;
// the O(n kl (kl+ku)) factorization and the triangular solves run in FP32, where
// GB300 has 74x the FP64 throughput.
//
// The solve is a sequence of launches, each shaped for its own bound:
//   factor   -- one group per system (a warp, or a CTA for wide bands): rounding,
//               FP32 LU, first solve.  Latency-bound column chains.
//   residual -- one CTA per system, one lane per row: the FP64 residual of up to
//               8 right-hand sides per pass over A, diagonal by diagonal, so every
//               lane of every DFMA does useful work.  Bounded by GB300's FP64 pipe
//               (1/74 of the FP32 rate), the cost this design minimises.
//   correct  -- one warp per system: the FP32 correction solve and X += d.
// `residual` and `correct` alternate maxit times; systems that have converged are
// skipped, and once every system has converged the launches return at once.
#include "lu.cuh"
#include "lureg.cuh"
#include "mixedlu.cuh"

namespace bm {

// Corrections per call at most (each is one correction and one residual launch).
constexpr int kMixedMaxCorrections = 100;

struct MixedParams {
  i64 count;
  const bm_gb_desc* descs;
  const int32_t* order;
  const double* AB;  // FP64 gbtrf storage, original matrix in rows kl.. (read only)
  const double* B;   // right-hand sides (read only)
  double* X;         // solutions (same layout as B)
  i64* ipiv;
  i64* info;
  float* AB32;       // FP32 factor storage (same offsets as AB)
  float* R32;        // FP32 residual / correction (leading dim n per system)
  int32_t* iters;    // per system: corrections so far (>= 0 while refining, -(k+1) once done)
  double* berr;      // per system: latest backward error (max over right-hand sides)
  int32_t* counter;  // 4 int32: work queues and converged-system counts of the two parities
  double tol;
  int maxit;
  i64 group_elems;   // shared-memory floats per warp (narrow factor part, correct)
  i64 wide_kl, wide_ku, narrow_kl, narrow_ku;  // band bounds the factor launch's shared memory was sized for
};

// A system whose descriptor is illegal or exceeds the launch's band bounds: info gets
// -(field number), and the system takes no factorization and no refinement.
__device__ __forceinline__ bool mixed_reject(const MixedParams& p, int s, i64 bkl, i64 bku, bool leader) {
  const i64 bad = desc_check(p.descs[s], bkl, bku);
  if (bad && leader) {
    p.info[s] = bad;
    p.iters[s] = -1;
    p.berr[s] = 0.0;
  }
  return bad != 0;
}

// ------------------------------------------------------------------ factor
template <int G>
__device__ void mixed_factor_system(const MixedParams& p, int s, float* smem) {
  constexpr int NT = Grp<G>::NT;
  const int tid = Grp<G>::tid(), wig = tid >> 5;
  auto sync = [] { Grp<G>::sync(); };
  const bm_gb_desc d = p.descs[s];
  const int kl = (int)d.kl, ku = (int)d.ku;
  const i64 n = d.n, ldab = d.ldab;
  const double* A = p.AB + d.ab_offset;
  float* A32 = p.AB32 + d.ab_offset;
  i64* ip = p.ipiv + d.ipiv_offset;
  // ---- round to FP32 (the top kl fill-in rows start at zero)
  {
    const i64 tot = ldab * n;
    i64 r = tid;  // row of element e within its column, advanced without division
    while (r >= ldab) r -= ldab;
    for (i64 e = tid; e < tot; e += NT) {
      A32[e] = r < kl ? 0.0f : (float)A[e];
      r += NT;
      while (r >= ldab) r -= ldab;
    }
  }
  sync();
  const bool regf = reg_fits<float>(kl, ku, NT);
  const i64 inf = regf ? gbtrf_reg_any<float, NT>(n, n, kl, ku, A32, ldab, ip, smem, tid, NT, G > 1)
                       : gbtrf_group<float, 4, G>(n, n, kl, ku, A32, ldab, ip, smem);
  sync();
  if (inf == 0) {
    const int nr = (int)d.nrhs;
    const double* Bs = p.B + d.b_offset;
    double* Xs = p.X + d.b_offset;
    float* Rs = p.R32 + d.b_offset;
    for (i64 e = tid; e < n * nr; e += NT) {
      const i64 c = e / n, i = e - c * n;
      Rs[e] = (float)Bs[i + c * d.ldb];
    }
    sync();
    if (reg_solve_fits<float>(kl, ku)) {
      if (wig == 0) gbtrs_reg_any<float, kMaxRhs>(n, kl, ku, nr, A32, ldab, ip, Rs, n, smem, tid & 31);
    } else {
      gbtrs_all<float, G>(false, n, kl, ku, nr, A32, ldab, ip, Rs, n, smem);
    }
    sync();
    for (i64 e = tid; e < n * nr; e += NT) {
      const i64 c = e / n, i = e - c * n;
      Xs[i + c * d.ldb] = (double)Rs[e];
    }
  }
  if (tid == 0) {
    p.info[s] = inf;
    p.iters[s] = inf == 0 ? 0 : -1;  // a singular FP32 factor: no refinement
    p.berr[s] = 0.0;
  }
  sync();
}

// Two-part schedule, as gbsv_batched_kernel: wide systems (order[0..n_wide)) one per
// CTA of W warps, then narrow systems one per warp in group_elems-float slices.
template <int W>
__global__ void __launch_bounds__(32 * W) mixed_factor_kernel(const MixedParams p, i64 n_wide) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* base = reinterpret_cast<float*>(smem_raw);
  int idx;
  for (;;) {
    idx = next_item<W>(p.counter, reinterpret_cast<int*>(base));
    if (idx >= n_wide) break;
    const int s = p.order ? p.order[idx] : idx;
    if (s < 0 || s >= p.count || mixed_reject(p, s, p.wide_kl, p.wide_ku, threadIdx.x == 0)) continue;
    mixed_factor_system<W>(p, s, base);
    __syncthreads();
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* ws = base + w * p.group_elems;
  int my = w == 0 ? idx : -1;
  for (;;) {
    if (my < 0) {
      int v = 0;
      if (lane == 0) v = atomicAdd(p.counter, 1);
      my = __shfl_sync(0xffffffffu, v, 0);
    }
    if (my >= p.count) break;
    const int s = p.order ? p.order[my] : my;
    my = -1;
    if (s < 0 || s >= p.count || mixed_reject(p, s, p.narrow_kl, p.narrow_ku, lane == 0)) continue;
    mixed_factor_system<1>(p, s, ws);
  }
}

// ------------------------------------------------------------------ residual
// One CTA of kResW warps per system.  Warp w takes the 32-row tiles w, w+kResW, ...;
// lane L owns row i = r0 + L and accumulates y_c(i) = sum_j A(i,j) x_c(j) over the
// diagonals d = j - i = -kl .. ku in ascending order (ascending j, as the row's terms
// of a gbmv), so every DFMA has all 32 lanes busy.  A tile's diagonals are staged in
// chunks of 32: A(i, i+d) for the tile's rows (each band column contributes one
// contiguous run, copied with coalesced cp.async into a skewed [d][row] layout) and
// the x window the chunk reads, double-buffered per warp.
constexpr int kResW = 8;    // warps per CTA
constexpr int kResNR = 8;   // right-hand sides per pass over A
constexpr int kResDC = 32;  // diagonals per staged chunk
struct ResWarpStage {
  double a[kResDC][32];          // a[dd][L] = A(r0+L, r0+L+d0+dd)
  double x[kResNR][2 * kResDC];  // x[c][k] = x_c(r0+d0+k)
};
constexpr int kResSmemBytes = kResW * 2 * (int)sizeof(ResWarpStage) + kResW * (3 * kResNR + 1) * 8 + 64;

// |a| of a double as a float, truncated to 20 mantissa bits, with integer operations
// only (GB300's FP64 pipe is the residual's bound; the row sums of |A| for ||A||_inf
// need no more than this accuracy).
__device__ __forceinline__ float abs_f32_of(double a) {
  const unsigned hi = (unsigned)__double2hiint(a) & 0x7fffffffu;
  const int e = (int)(hi >> 20) - 1023 + 127;
  if (e <= 0) return 0.0f;
  if (e >= 255) return __int_as_float(0x7f800000);
  return __uint_as_float(((unsigned)e << 23) | ((hi & 0xfffffu) << 3));
}

__device__ __forceinline__ double nan_max(double a, double b) { return (b > a || b != b) ? b : a; }
// nan_max for non-negative a and b (absolute values): their IEEE bit patterns order as
// the values do, with every NaN above infinity, so the maximum is an unsigned integer
// comparison and stays off the FP64 pipe (two FP64 compares here would cost about as
// much as two of the residual's fmas).
__device__ __forceinline__ double nan_max_abs(double a, double b) {
  const unsigned long long ua = (unsigned long long)__double_as_longlong(a);
  const unsigned long long ub = (unsigned long long)__double_as_longlong(b);
  return ub > ua ? b : a;
}
__device__ __forceinline__ float nan_maxf(float a, float b) { return (b > a || b != b) ? b : a; }

// The tiles of one warp for right-hand sides [c0, c0+NR): residuals into R32 and the
// lane's running maxima of |r|, |x|, |b| per right-hand side and of the |A| row sums.
template <int NR>
__device__ void residual_tiles(const MixedParams& p, const bm_gb_desc& d, int c0, ResWarpStage* st, int w, int lane,
                               double* rn, double* xn, double* bn, float& an) {
  const i64 n = d.n, ldab = d.ldab, ldb = d.ldb;
  const int kl = (int)d.kl, ku = (int)d.ku;
  const double* A = p.AB + d.ab_offset;
  const double* Bs = p.B + d.b_offset + (i64)c0 * ldb;
  const double* Xs = p.X + d.b_offset + (i64)c0 * ldb;
  float* Rs = p.R32 + d.b_offset + (i64)c0 * n;
  const i64 ntiles = (n + 31) >> 5;
  const int nch = (kl + ku + kResDC) / kResDC;  // chunks of diagonals per tile
  const i64 my_tiles = ntiles > w ? (ntiles - 1 - w) / kResW + 1 : 0;
  const i64 items = my_tiles * nch;
  auto stage = [&](i64 q) {
    ResWarpStage& S = st[q & 1];
    const i64 r0 = ((i64)w + (q / nch) * kResW) << 5;
    const int d0 = -kl + (int)(q % nch) * kResDC;
    // A: band column j = r0 + d0 + t holds A(i, j) for rows i = r0 + L with
    // d = j - i in [d0, d0 + 32); the lanes of one t read one contiguous run
    for (int t = 0; t < 2 * kResDC - 1; ++t) {
      const int dd = t - lane;
      if (dd >= 0 && dd < kResDC) {
        const i64 j = r0 + d0 + t, i = r0 + lane;
        const int dg = d0 + dd;
        const bool ok = dg <= ku && i < n && j >= 0 && j < n;
        cp_async_elem(&S.a[dd][lane], ok ? A + (kl + ku - dg) + j * ldab : A, ok);
      }
    }
#pragma unroll
    for (int c = 0; c < NR; ++c)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const i64 xi = r0 + d0 + lane + 32 * h;
        const bool ok = xi >= 0 && xi < n;
        cp_async_elem(&S.x[c][lane + 32 * h], ok ? Xs + xi + c * ldb : Xs, ok);
      }
    cp_async_commit();
  };
  double y[NR];
#pragma unroll
  for (int c = 0; c < NR; ++c) y[c] = 0.0;
  float sabs = 0.0f;
  if (items > 0) stage(0);
  for (i64 q = 0; q < items; ++q) {
    if (q + 1 < items) {
      stage(q + 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncwarp();
    const ResWarpStage& S = st[q & 1];
    const int ch = (int)(q % nch);
    const int d0 = -kl + ch * kResDC;
    const int ndd = min(kResDC, ku - d0 + 1);
#pragma unroll 4
    for (int dd = 0; dd < ndd; ++dd) {
      const double a = S.a[dd][lane];
      sabs += abs_f32_of(a);
#pragma unroll
      for (int c = 0; c < NR; ++c) y[c] = fma(a, S.x[c][lane + dd], y[c]);
    }
    __syncwarp();  // the buffer is restaged two items later
    if (ch == nch - 1) {  // the tile is complete
      const i64 i = (((i64)w + (q / nch) * kResW) << 5) + lane;
      if (i < n) {
#pragma unroll
        for (int c = 0; c < NR; ++c) {
          const double b = Bs[i + c * ldb], x = Xs[i + c * ldb];
          const double r = b - y[c];
          Rs[i + (i64)c * n] = (float)r;
          rn[c] = nan_max_abs(rn[c], fabs(r));
          xn[c] = nan_max_abs(xn[c], fabs(x));
          bn[c] = nan_max_abs(bn[c], fabs(b));
        }
        an = nan_maxf(an, sabs);
      }
#pragma unroll
      for (int c = 0; c < NR; ++c) y[c] = 0.0;
      sabs = 0.0f;
    }
  }
}

template <int NR>
__device__ double residual_group(const MixedParams& p, const bm_gb_desc& d, int c0, ResWarpStage* st, double* red) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double rn[NR], xn[NR], bn[NR];
#pragma unroll
  for (int c = 0; c < NR; ++c) rn[c] = xn[c] = bn[c] = 0.0;
  float an = 0.0f;
  residual_tiles<NR>(p, d, c0, st, w, lane, rn, xn, bn, an);
  // warp, then CTA maxima (NaN propagates)
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
#pragma unroll
    for (int c = 0; c < NR; ++c) {
      rn[c] = nan_max_abs(rn[c], __shfl_xor_sync(0xffffffffu, rn[c], off));
      xn[c] = nan_max_abs(xn[c], __shfl_xor_sync(0xffffffffu, xn[c], off));
      bn[c] = nan_max_abs(bn[c], __shfl_xor_sync(0xffffffffu, bn[c], off));
    }
    an = nan_maxf(an, __shfl_xor_sync(0xffffffffu, an, off));
  }
  double* rw = red + w * (3 * kResNR + 1);
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < NR; ++c) {
      rw[c] = rn[c];
      rw[kResNR + c] = xn[c];
      rw[2 * kResNR + c] = bn[c];
    }
    rw[3 * kResNR] = (double)an;
  }
  __syncthreads();
  double be = 0.0;
  if (threadIdx.x == 0) {
    double anorm = red[3 * kResNR];
    for (int k = 1; k < kResW; ++k) anorm = nan_max(anorm, red[k * (3 * kResNR + 1) + 3 * kResNR]);
    for (int c = 0; c < NR; ++c) {
      double r = red[c], x = red[kResNR + c], b = red[2 * kResNR + c];
      for (int k = 1; k < kResW; ++k) {
        const double* rk = red + k * (3 * kResNR + 1);
        r = nan_max(r, rk[c]);
        x = nan_max(x, rk[kResNR + c]);
        b = nan_max(b, rk[2 * kResNR + c]);
      }
      const double den = anorm * x + b;
      const double bc = den > 0.0 ? r / den : r;
      be = nan_max(be, bc);
    }
  }
  __syncthreads();
  return be;  // meaningful in thread 0
}

// Pass k of the refinement (parity par = k & 1): queue counter[2 par], systems still
// refining after the pass counted in counter[2 par + 1], systems refining after the
// previous pass read from counter[2 (1 - par) + 1] (zero: nothing to do).
__global__ void __launch_bounds__(32 * kResW, 1) mixed_residual_kernel(const MixedParams p, int par) {
  if (*reinterpret_cast<volatile const int32_t*>(p.counter + 2 * (1 - par) + 1) == 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ResWarpStage* st = reinterpret_cast<ResWarpStage*>(smem_raw) + 2 * (threadIdx.x >> 5);
  double* red = reinterpret_cast<double*>(smem_raw + kResW * 2 * sizeof(ResWarpStage));
  int* hdr = reinterpret_cast<int*>(red + kResW * (3 * kResNR + 1));
  int32_t* queue = p.counter + 2 * par;
  for (;;) {
    if (threadIdx.x == 0) hdr[0] = atomicAdd(queue, 1);
    __syncthreads();
    const int idx = hdr[0];
    __syncthreads();
    if (idx >= p.count) break;
    const int s = p.order ? p.order[idx] : idx;
    if (s < 0 || s >= p.count) continue;
    const int it = p.iters[s];
    if (it < 0) continue;  // converged, or no FP32 factor
    const bm_gb_desc d = p.descs[s];
    double be = 0.0;
    for (int c0 = 0; c0 < (int)d.nrhs; c0 += kResNR) {
      const int nr = (int)min((i64)kResNR, d.nrhs - c0);
      double b;
      switch (nr) {
        case 1: b = residual_group<1>(p, d, c0, st, red); break;
        case 2: b = residual_group<2>(p, d, c0, st, red); break;
        case 3: b = residual_group<3>(p, d, c0, st, red); break;
        case 4: b = residual_group<4>(p, d, c0, st, red); break;
        case 5: b = residual_group<5>(p, d, c0, st, red); break;
        case 6: b = residual_group<6>(p, d, c0, st, red); break;
        case 7: b = residual_group<7>(p, d, c0, st, red); break;
        default: b = residual_group<8>(p, d, c0, st, red); break;
      }
      be = nan_max(be, b);
    }
    if (threadIdx.x == 0) {
      p.berr[s] = be;
      if (!(be > p.tol) || it >= p.maxit) p.iters[s] = -(it + 1);  // NaN stops too
      else atomicAdd(queue + 1, 1);
    }
  }
}

// ------------------------------------------------------------------ correct
// Correction k (parity par = k & 1): one warp per system still refining solves
// LU32 d = r in place in R32 and adds d to X in FP64.
template <int W>
__global__ void __launch_bounds__(32 * W) mixed_correct_kernel(const MixedParams p, int par) {
  if (*reinterpret_cast<volatile const int32_t*>(p.counter + 2 * (1 - par) + 1) == 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* ws = reinterpret_cast<float*>(smem_raw) + w * p.group_elems;
  int32_t* queue = p.counter + 2 * par;
  for (;;) {
    int v = 0;
    if (lane == 0) v = atomicAdd(queue, 1);
    v = __shfl_sync(0xffffffffu, v, 0);
    if (v >= p.count) break;
    const int s = p.order ? p.order[v] : v;
    if (s < 0 || s >= p.count || p.iters[s] < 0) continue;
    const bm_gb_desc d = p.descs[s];
    const int kl = (int)d.kl, ku = (int)d.ku, nr = (int)d.nrhs;
    const i64 n = d.n;
    const float* A32 = p.AB32 + d.ab_offset;
    const i64* ip = p.ipiv + d.ipiv_offset;
    float* Rs = p.R32 + d.b_offset;
    double* Xs = p.X + d.b_offset;
    if (reg_solve_fits<float>(kl, ku)) gbtrs_reg_any<float, kMaxRhs>(n, kl, ku, nr, A32, d.ldab, ip, Rs, n, ws, lane);
    else gbtrs_all<float, 1>(false, n, kl, ku, nr, A32, d.ldab, ip, Rs, n, ws);
    __syncwarp();
    for (i64 e = lane; e < n * nr; e += 32) {
      const i64 c = e / n, i = e - c * n;
      Xs[i + c * d.ldb] += (double)Rs[e];
    }
    if (lane == 0) p.iters[s] += 1;
    __syncwarp();
  }
}

// iters: -(k+1) (done after k corrections) -> k
__global__ void mixed_finish_kernel(i64 count, int32_t* iters) {
  for (i64 s = blockIdx.x * (i64)blockDim.x + threadIdx.x; s < count; s += (i64)gridDim.x * blockDim.x) {
    const int v = iters[s];
    iters[s] = v < 0 ? -v - 1 : v;
  }
}

// ------------------------------------------------------------------ blocked path
// Bands with kl <= 80 and kl + ku <= 151 (and a window that fits shared memory): the
// blocked FP32 LU by one CTA per system and the warp solves of mixedlu.cuh.
__global__ void __launch_bounds__(kBlkThreads, 4) mixed_lu_blocked_kernel(const MixedParams p, int stage) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int* q = reinterpret_cast<int*>(smem_raw + 80);  // the next system (header bytes 80..83)
  for (;;) {
    if (threadIdx.x == 0) *q = atomicAdd(p.counter, 1);
    __syncthreads();
    const int idx = *q;
    __syncthreads();
    if (idx >= p.count) break;
    const int s = p.order ? p.order[idx] : idx;
    if (s < 0 || s >= p.count || mixed_reject(p, s, p.wide_kl, p.wide_ku, threadIdx.x == 0)) continue;
    const bm_gb_desc d = p.descs[s];
    const i64 inf = blk_lu_cta(d.n, (int)d.kl, (int)d.ku, p.AB + d.ab_offset, d.ldab, p.AB32 + d.ab_offset, d.ldab,
                               p.ipiv + d.ipiv_offset, smem_raw, stage != 0);
    if (threadIdx.x == 0) {
      p.info[s] = inf;
      p.iters[s] = inf == 0 ? 0 : -1;  // a singular FP32 factor: no refinement
      p.berr[s] = 0.0;
    }
  }
}

// Work item q of a solve launch: system order[q mod count], right-hand sides
// [0, 4) for q < count and [4, nrhs) for the rest (4 at a time), one warp each.
// first != 0: the first solve, X = FP64(LU32 \ FP32(B)); else correction k (parity
// par): LU32 d = r in place in R32 and X += d, for the systems still refining.
template <int W>
__global__ void __launch_bounds__(32 * W, 16 / W) mixed_solve_blocked_kernel(const MixedParams p, int par, int first) {
  if (!first && *reinterpret_cast<volatile const int32_t*>(p.counter + 2 * (1 - par) + 1) == 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  float* ring = reinterpret_cast<float*>(smem_raw) + (threadIdx.x >> 5) * kSolveRingFloats;
  int32_t* queue = p.counter + 2 * par;
  for (;;) {
    int v = 0;
    if (lane == 0) v = atomicAdd(queue, 1);
    v = __shfl_sync(0xffffffffu, v, 0);
    if (v >= 2 * p.count) break;
    const bool tail = v >= p.count;
    const int s = p.order ? p.order[tail ? v - p.count : v] : (tail ? v - (int)p.count : v);
    if (s < 0 || s >= p.count || p.iters[s] < 0) continue;
    const bm_gb_desc d = p.descs[s];
    const i64 n = d.n, nrhs = d.nrhs;
    if (tail && nrhs <= kSolveNR) continue;
    if (!first && !tail && lane == 0) p.iters[s] += 1;
    for (i64 c0 = tail ? kSolveNR : 0; c0 < (tail ? nrhs : min((i64)kSolveNR, nrhs)); c0 += kSolveNR) {
      const int nr = (int)min((i64)kSolveNR, nrhs - c0);
      float* Rs = p.R32 + d.b_offset + c0 * n;
      double* Xs = p.X + d.b_offset + c0 * d.ldb;
      if (first) {
        const double* Bs = p.B + d.b_offset + c0 * d.ldb;
        for (int c = 0; c < nr; ++c)
          for (i64 i = lane; i < n; i += 32) Rs[i + c * n] = (float)Bs[i + c * d.ldb];
        __syncwarp();
      }
      blk_solve_warp(n, (int)d.kl, (int)d.ku, nr, p.AB32 + d.ab_offset, d.ldab, p.ipiv + d.ipiv_offset, Rs, n, ring,
                     lane);
      __syncwarp();
      for (int c = 0; c < nr; ++c)
        for (i64 i = lane; i < n; i += 32) {
          const double r = (double)Rs[i + c * n];
          if (first) Xs[i + c * d.ldb] = r;
          else Xs[i + c * d.ldb] += r;
        }
      __syncwarp();
    }
  }
}

static int mixed_launch_blocked(MixedParams p, i64 kl_max, i64 ku_max, cudaStream_t stream, const char* name) {
  constexpr int SW = 4;  // warps per CTA of the solve kernel
  // the cp.async staging of window slides, unless it costs an SM a CTA
  int lper = 0, lper_ns = 0, r;
  const int bytes_s = (int)blk_smem_bytes(kl_max, ku_max, true), bytes_ns = (int)blk_smem_bytes(kl_max, ku_max, false);
  if ((r = cuda_status(ensure_smem((const void*)mixed_lu_blocked_kernel, std::min(bytes_s, 227 * 1024)), name)))
    return r;
  if (bytes_s <= 227 * 1024 &&
      (r = cuda_status(
           cudaOccupancyMaxActiveBlocksPerMultiprocessor(&lper, mixed_lu_blocked_kernel, kBlkThreads, bytes_s), name)))
    return r;
  if ((r = cuda_status(
           cudaOccupancyMaxActiveBlocksPerMultiprocessor(&lper_ns, mixed_lu_blocked_kernel, kBlkThreads, bytes_ns),
           name)))
    return r;
  const bool stage = lper > 0 && lper >= lper_ns;
  const int lbytes = stage ? bytes_s : bytes_ns;
  lper = stage ? lper : lper_ns;
  const i64 lgrid = std::min<i64>((i64)num_sms() * std::max(lper, 1), p.count);
  const int sbytes = SW * kSolveRingFloats * (int)sizeof(float);
  if ((r = cuda_status(ensure_smem((const void*)mixed_solve_blocked_kernel<SW>, sbytes), name))) return r;
  int sper = 0;
  if ((r = cuda_status(
           cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sper, mixed_solve_blocked_kernel<SW>, 32 * SW, sbytes), name)))
    return r;
  const i64 sgrid = std::min<i64>((i64)num_sms() * std::max(sper, 1), ceil_div(2 * p.count, (i64)SW));
  if ((r = cuda_status(ensure_smem((const void*)mixed_residual_kernel, kResSmemBytes), name))) return r;
  const i64 rgrid = std::min<i64>((i64)num_sms(), p.count);

  // counter[3] != 0: the first residual pass has work
  if ((r = cuda_status(cudaMemsetAsync(p.counter, 0, 4 * sizeof(int32_t), stream), name))) return r;
  if ((r = cuda_status(cudaMemsetAsync(reinterpret_cast<char*>(p.counter + 3), 1, 1, stream), name))) return r;
  mixed_lu_blocked_kernel<<<(unsigned)lgrid, kBlkThreads, lbytes, stream>>>(p, stage ? 1 : 0);
  if ((r = launch_status(name))) return r;
  mixed_solve_blocked_kernel<SW><<<(unsigned)sgrid, 32 * SW, sbytes, stream>>>(p, 1, 1);  // queue counter[2]
  if ((r = launch_status(name))) return r;
  for (int k = 0; k <= p.maxit; ++k) {
    const int par = k & 1;
    if (k > 0) {
      if ((r = cuda_status(cudaMemsetAsync(p.counter + 2 * par, 0, sizeof(int32_t), stream), name))) return r;
      mixed_solve_blocked_kernel<SW><<<(unsigned)sgrid, 32 * SW, sbytes, stream>>>(p, par, 0);
      if ((r = launch_status(name))) return r;
    }
    if ((r = cuda_status(cudaMemsetAsync(p.counter + 2 * par, 0, 2 * sizeof(int32_t), stream), name))) return r;
    mixed_residual_kernel<<<(unsigned)rgrid, 32 * kResW, kResSmemBytes, stream>>>(p, par);
    if ((r = launch_status(name))) return r;
  }
  mixed_finish_kernel<<<(unsigned)std::min<i64>(ceil_div(p.count, 256), 1024), 256, 0, stream>>>(p.count, p.iters);
  return launch_status(name);
}

// Floats of one group's shared memory for systems up to (kl, ku): FP32 factor window
// and solve staging; 0 when the refined solve does not support the band.
template <int NLMAX>
static i64 mixed_group_elems(i64 kl, i64 ku) {
  if (kl + ku > 256) return 0;
  const i64 fac = gbtrf_smem_elems<4>((int)kl, (int)ku);
  const i64 reg = (reg_group_bytes<float, NLMAX, kMaxRhs>(kl, ku) + 3) / 4;
  const i64 f = std::max(std::max(std::max(fac, gbtrs_smem_elems((int)kl, (int)ku)), (i64)(kHdr + 16)), reg);
  return ((f + 3) / 4) * 4;
}

template <int W>
static int mixed_launch(MixedParams p, const bm_gb_schedule& sc, cudaStream_t stream, const char* name) {
  const i64 we = sc.n_wide > 0 ? mixed_group_elems<32 * W>(sc.wide_kl, sc.wide_ku) : 1;
  const i64 ne = sc.n_wide < p.count ? mixed_group_elems<32>(sc.narrow_kl, sc.narrow_ku) : 1;
  if (we == 0 || ne == 0) {
    set_error("%s: kl + ku exceeds the refined solve's limit of 256", name);
    return BM_ERR_UNSUPPORTED;
  }
  // ---- factor
  p.group_elems = sc.n_wide < p.count ? ne : 0;
  const i64 bytes = std::max(std::max(we, W * (sc.n_wide < p.count ? ne : 0)), (i64)kHdr) * 4;
  if (bytes > 227 * 1024) {
    set_error("%s: the schedule's shared memory (%lld bytes) exceeds the per-CTA limit", name, (long long)bytes);
    return BM_ERR_UNSUPPORTED;
  }
  const void* kfn = (const void*)mixed_factor_kernel<W>;
  int r = cuda_status(ensure_smem(kfn, (int)bytes), name);
  if (r) return r;
  int per_sm = 0;
  r = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mixed_factor_kernel<W>, 32 * W, (int)bytes),
                  name);
  if (r) return r;
  per_sm = std::max(per_sm, 1);
  const i64 need = sc.n_wide + ceil_div(p.count - sc.n_wide, (i64)W);
  const i64 grid = std::min<i64>((i64)num_sms() * per_sm, std::max<i64>(need, 1));
  // counter[3] != 0: the first residual pass has work
  if ((r = cuda_status(cudaMemsetAsync(p.counter, 0, 4 * sizeof(int32_t), stream), name))) return r;
  if ((r = cuda_status(cudaMemsetAsync(reinterpret_cast<char*>(p.counter + 3), 1, 1, stream), name))) return r;
  mixed_factor_kernel<W><<<(unsigned)grid, 32 * W, (int)bytes, stream>>>(p, sc.n_wide);
  if ((r = launch_status(name))) return r;

  // ---- correction solves: one warp per system, W warps per CTA
  const i64 kl_all = std::max(sc.n_wide > 0 ? sc.wide_kl : 0, sc.n_wide < p.count ? sc.narrow_kl : 0);
  const i64 ku_all = std::max(sc.n_wide > 0 ? sc.wide_ku : 0, sc.n_wide < p.count ? sc.narrow_ku : 0);
  const i64 ce = std::max(mixed_group_elems<32>(kl_all, ku_all), (i64)kHdr);
  const int cbytes = (int)(W * ce * 4);
  if (cbytes > 227 * 1024) {
    set_error("%s: the correction's shared memory (%d bytes) exceeds the per-CTA limit", name, cbytes);
    return BM_ERR_UNSUPPORTED;
  }
  if ((r = cuda_status(ensure_smem((const void*)mixed_correct_kernel<W>, cbytes), name))) return r;
  int cper = 0;
  if ((r = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cper, mixed_correct_kernel<W>, 32 * W, cbytes),
                       name)))
    return r;
  const i64 cgrid = std::min<i64>((i64)num_sms() * std::max(cper, 1), std::max<i64>(ceil_div(p.count, (i64)W), 1));
  // ---- residual passes: one CTA per system
  if ((r = cuda_status(ensure_smem((const void*)mixed_residual_kernel, kResSmemBytes), name))) return r;
  const i64 rgrid = std::min<i64>((i64)num_sms(), std::max<i64>(p.count, 1));

  for (int k = 0; k <= p.maxit; ++k) {
    const int par = k & 1;
    if (k > 0) {
      MixedParams q = p;
      q.group_elems = ce;
      if ((r = cuda_status(cudaMemsetAsync(p.counter + 2 * par, 0, sizeof(int32_t), stream), name))) return r;
      mixed_correct_kernel<W><<<(unsigned)cgrid, 32 * W, cbytes, stream>>>(q, par);
      if ((r = launch_status(name))) return r;
    }
    if ((r = cuda_status(cudaMemsetAsync(p.counter + 2 * par, 0, 2 * sizeof(int32_t), stream), name))) return r;
    mixed_residual_kernel<<<(unsigned)rgrid, 32 * kResW, kResSmemBytes, stream>>>(p, par);
    if ((r = launch_status(name))) return r;
  }
  mixed_finish_kernel<<<(unsigned)std::min<i64>(ceil_div(std::max<i64>(p.count, 1), 256), 1024), 256, 0, stream>>>(
      p.count, p.iters);
  return launch_status(name);
}

static int dsgbsv_batched_impl(const MixedParams& p, const bm_gb_schedule* sc, cudaStream_t stream, const char* name) {
  if (p.count < 0) return -1;
  if (!p.descs && p.count) return -2;
  if (!sc || sc->n_wide < 0 || sc->n_wide > p.count || (sc->warps != 4 && sc->warps != 8) || sc->wide_kl < 0 ||
      sc->wide_ku < 0 || sc->narrow_kl < 0 || sc->narrow_ku < 0)
    return -4;
  if (!p.counter) return -14;
  if (!(p.tol >= 0.0)) return -15;
  if (p.maxit < 0) return -16;
  if (p.count == 0) return BM_OK;
  const i64 kl_all = std::max(sc->n_wide > 0 ? sc->wide_kl : 0, sc->n_wide < p.count ? sc->narrow_kl : 0);
  const i64 ku_all = std::max(sc->n_wide > 0 ? sc->wide_ku : 0, sc->n_wide < p.count ? sc->narrow_ku : 0);
  MixedParams q = p;
  if (blk_lu_fits(kl_all, ku_all) && blk_solve_fits(kl_all, ku_all) &&
      blk_smem_bytes(kl_all, ku_all, false) <= 227 * 1024) {
    q.wide_kl = q.narrow_kl = kl_all;  // one CTA per system, sized for the widest band
    q.wide_ku = q.narrow_ku = ku_all;
    return mixed_launch_blocked(q, kl_all, ku_all, stream, name);
  }
  q.wide_kl = sc->wide_kl;
  q.wide_ku = sc->wide_ku;
  q.narrow_kl = sc->narrow_kl;
  q.narrow_ku = sc->narrow_ku;
  if (sc->warps == 8) return mixed_launch<8>(q, *sc, stream, name);
  return mixed_launch<4>(q, *sc, stream, name);
}

}  // namespace bm

// Arguments are checked in order, LAPACK style (-i for argument i), before any CUDA
// call; `order` may be NULL (natural order), and the band, right-hand-side and pivot
// buffers may be NULL when they are empty.
extern "C" int bm_dsgbsv_batched(int64_t count, const bm_gb_desc* descs, const int32_t* order, const double* AB,
                                 const double* B, double* X, int64_t* ipiv, int64_t* info, float* AB32, float* R32,
                                 int32_t* iters, double* berr, int32_t* counter, double tol, int64_t maxit,
                                 int64_t max_kl, int64_t max_ku, bm_stream_t stream) {
  if (count < 0) return -1;
  if (count > 0) {  // the per-system arrays (the others may be empty: all n or nrhs zero)
    if (!descs) return -2;
    if (!info) return -8;
    if (!iters) return -11;
    if (!berr) return -12;
  }
  if (!counter) return -13;
  if (!(tol >= 0.0)) return -14;
  if (maxit < 0) return -15;
  if (max_kl < 0) return -16;
  if (max_ku < 0) return -17;
  bm::MixedParams p;
  p.count = count; p.descs = descs; p.order = order; p.AB = AB; p.B = B; p.X = X; p.ipiv = ipiv; p.info = info;
  p.AB32 = AB32; p.R32 = R32; p.iters = iters; p.berr = berr; p.counter = counter; p.tol = tol;
  p.maxit = (int)std::min<int64_t>(maxit, bm::kMixedMaxCorrections);
  p.group_elems = 0;
  bm_gb_schedule sc;  // every system wide (4 warps) once the widest window holds 512 entries, else narrow
  sc.n_wide = (max_kl + 1) * (max_kl + max_ku + 1) >= 512 ? count : 0;
  sc.warps = 4;
  sc.wide_kl = sc.narrow_kl = max_kl;
  sc.wide_ku = sc.narrow_ku = max_ku;
  return bm::dsgbsv_batched_impl(p, &sc, reinterpret_cast<cudaStream_t>(stream), "bm_dsgbsv_batched");
}

extern "C" int bm_dsgbsv_batched_sched(int64_t count, const bm_gb_desc* descs, const int32_t* order,
                                       const bm_gb_schedule* sched, const double* AB, const double* B, double* X,
                                       int64_t* ipiv, int64_t* info, float* AB32, float* R32, int32_t* iters,
                                       double* berr, int32_t* counter, double tol, int64_t maxit, bm_stream_t stream) {
  if (count < 0) return -1;
  if (count > 0 && !descs) return -2;
  if (!sched || sched->n_wide < 0 || sched->n_wide > count || (sched->warps != 4 && sched->warps != 8) ||
      sched->wide_kl < 0 || sched->wide_ku < 0 || sched->narrow_kl < 0 || sched->narrow_ku < 0)
    return -4;
  if (count > 0) {  // the per-system arrays (the others may be empty: all n or nrhs zero)
    if (!info) return -9;
    if (!iters) return -12;
    if (!berr) return -13;
  }
  if (!counter) return -14;
  if (!(tol >= 0.0)) return -15;
  if (maxit < 0) return -16;
  bm::MixedParams p;
  p.count = count; p.descs = descs; p.order = order; p.AB = AB; p.B = B; p.X = X; p.ipiv = ipiv; p.info = info;
  p.AB32 = AB32; p.R32 = R32; p.iters = iters; p.berr = berr; p.counter = counter; p.tol = tol;
  p.maxit = (int)std::min<int64_t>(maxit, bm::kMixedMaxCorrections);
  p.group_elems = 0;
  return bm::dsgbsv_batched_impl(p, sched, reinterpret_cast<cudaStream_t>(stream), "bm_dsgbsv_batched_sched");
}
