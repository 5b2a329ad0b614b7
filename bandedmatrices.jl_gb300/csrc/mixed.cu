// Mixed-precision refined banded solves (no counterpart in the reference; the
// spec addition beside lu!/ldiv!, src/banded/BandedLU.jl:90-103,
// src/banded/linalg.jl:24-30).
//
// Per system (one warp): the FP64 band A is rounded to an FP32 copy in gbtrf
// storage and factored in FP32 with partial pivoting (the same warp algorithm as
// the FP64 path, lu.cuh).  Then, for each right-hand side b,
//     x = FP64(LU32 \ FP32(b))
//     repeat: r = b - A x            (FP64, from the original FP64 band)
//             berr = ||r||_inf / (||A||_inf ||x||_inf + ||b||_inf)
//             stop when berr <= tol or after maxit corrections
//             x = x + FP64(LU32 \ FP32(r))
// The residual and the update, the steps whose stability needs it, run in FP64;
// the O(n kl (kl+ku)) factorization and the triangular solves run in FP32, where
// GB300 has 64x the FP64 throughput.
#include "lu.cuh"
#include "lureg.cuh"

namespace bm {

// R = B - A X on rows [rb, re) for up to kResRhs right-hand sides of one system,
// written to R32 (FP32, leading dim n); returns this warp's partial maxima of |r_c|,
// |x_c| (over the columns it read) and, with want_anorm, of the |A| row sums.  Each
// lane owns window rows w = lane + 32q (q < kResQ) in registers; band columns are
// streamed once per 32-column chunk, every lane reading the entry of its own row (a
// coalesced read of the column), so no shared memory and no synchronisation are
// needed.  Row i accumulates its terms in ascending column order.
constexpr int kResRhs = 4;
constexpr int kResQ = 5;      // window rows 32*Q >= 32 + kl + ku: Q = 5 for kl + ku <= 128,
constexpr int kResQWide = 9;  // Q = 9 for kl + ku <= 256 (chosen per launch)

template <int kResQ>
__device__ void residual_rows(i64 n, i64 rb, i64 re, int kl, int ku, int nr, const double* __restrict__ band,
                              i64 ldab, const double* __restrict__ B, const double* __restrict__ X, i64 ld,
                              float* __restrict__ R32, bool want_anorm, double& anorm, double* rnorm,
                              double* xnorm) {
  const int lane = threadIdx.x & 31;
  const int kv = kl + ku;  // band: A(i,j) = band[(ku + i - j) + j*ldab]
  double Y[kResQ][kResRhs], S[kResQ];
#pragma unroll
  for (int q = 0; q < kResQ; ++q) {
    S[q] = 0.0;
#pragma unroll
    for (int c = 0; c < kResRhs; ++c) Y[q][c] = 0.0;
  }
  double rn[kResRhs], xn[kResRhs], an = 0.0;
#pragma unroll
  for (int c = 0; c < kResRhs; ++c) rn[c] = xn[c] = 0.0;

  auto emit = [&](int q, i64 i) {
    if (i < rb || i >= re) return;
#pragma unroll
    for (int c = 0; c < kResRhs; ++c)
      if (c < nr) {
        const double ri = B[i + c * ld] - Y[q][c];
        R32[i + c * n] = (float)ri;
        rn[c] = fmax(rn[c], fabs(ri));
      }
    an = fmax(an, S[q]);
  };

  const i64 cb = max((i64)0, rb - kl), ce = min(n, re + ku);
  for (i64 j0 = cb; j0 < ce; j0 += 32) {
    const int jn = (int)min((i64)32, ce - j0);
    // window row w <-> matrix row j0 - ku + w;  column j0 + t touches w = t .. t + kv
    for (int t = 0; t < jn; ++t) {
      const i64 j = j0 + t;
      const double* col = band + j * ldab;
      double xj[kResRhs];
#pragma unroll
      for (int c = 0; c < kResRhs; ++c) {
        xj[c] = c < nr ? X[j + c * ld] : 0.0;
        xn[c] = fmax(xn[c], fabs(xj[c]));
      }
#pragma unroll
      for (int q = 0; q < kResQ; ++q) {
        const int r = lane + 32 * q - t;  // band row for this lane's window row
        const i64 i = j0 - ku + lane + 32 * q;
        if (r >= 0 && r <= kv && i >= 0 && i < n) {
          const double a = col[r];
#pragma unroll
          for (int c = 0; c < kResRhs; ++c) Y[q][c] = fma(a, xj[c], Y[q][c]);
          if (want_anorm) S[q] += fabs(a);
        }
      }
    }
    if (j0 + 32 < ce) {
      emit(0, j0 - ku + lane);  // rows j0-ku .. j0-ku+31 are complete
#pragma unroll
      for (int q = 0; q < kResQ - 1; ++q) {
        S[q] = S[q + 1];
#pragma unroll
        for (int c = 0; c < kResRhs; ++c) Y[q][c] = Y[q + 1][c];
      }
      S[kResQ - 1] = 0.0;
#pragma unroll
      for (int c = 0; c < kResRhs; ++c) Y[kResQ - 1][c] = 0.0;
    } else {
#pragma unroll
      for (int q = 0; q < kResQ; ++q) emit(q, j0 - ku + lane + 32 * q);
    }
  }
  for (int c = 0; c < kResRhs; ++c) {
    rnorm[c] = rn[c];
    xnorm[c] = xn[c];
  }
  anorm = an;
}

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
  float* R32;        // FP32 work copy of B's layout (leading dim n per system)
  int32_t* iters;    // per system: corrections taken (max over right-hand sides)
  double* berr;      // per system: final backward error (max over right-hand sides)
  int32_t* counter;
  double tol;
  int maxit;
  i64 group_elems;   // shared-memory floats per group
};

// One system of the batch (index s) by a group of G warps in `smem`; Q sizes the
// residual's register window.
template <int G, int Q>
__device__ void dsgbsv_system(const MixedParams& p, int s, float* smem) {
  constexpr int NT = Grp<G>::NT;
  const int tid = Grp<G>::tid(), wig = tid >> 5;
  double* red = reinterpret_cast<double*>(smem + kHdr);  // reduction scratch (between phases)
  auto sync = [] { Grp<G>::sync(); };
  {
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
    // ---- FP32 factorization: the register window where the band fits the group
    const bool regf = reg_fits<float>(kl, ku, NT);
    const bool regs = reg_solve_fits<float>(kl, ku);
    const i64 inf = regf ? gbtrf_reg_any<float, NT>(n, n, kl, ku, A32, ldab, ip, smem, tid, NT, G > 1)
                         : gbtrf_group<float, 4, G>(n, n, kl, ku, A32, ldab, ip, smem);
    sync();
    auto solve32 = [&](int nr, float* R) {
      if (regs) {
        if (wig == 0) gbtrs_reg_any<float, kMaxRhs>(n, kl, ku, nr, A32, ldab, ip, R, n, smem, tid & 31);
      } else {
        gbtrs_all<float, G>(false, n, kl, ku, nr, A32, ldab, ip, R, n, smem);
      }
    };
    if (tid == 0) p.info[s] = inf;
    int its_max = 0;
    double berr_max = 0.0;
    if (inf == 0) {
      const int nr_all = (int)d.nrhs;
      const double* Bs = p.B + d.b_offset;
      double* Xs = p.X + d.b_offset;
      float* Rs = p.R32 + d.b_offset;  // FP32 copy of B's layout (leading dim n)
      // x0 = LU32 \ b  for every right-hand side
      for (i64 e = tid; e < n * nr_all; e += NT) {
        const i64 c = e / n, i = e - c * n;
        Rs[e] = (float)Bs[i + c * d.ldb];
      }
      sync();
      solve32(nr_all, Rs);
      sync();
      for (i64 e = tid; e < n * nr_all; e += NT) {
        const i64 c = e / n, i = e - c * n;
        Xs[i + c * d.ldb] = (double)Rs[e];
      }
      sync();
      double anorm = -1.0;  // ||A||_inf, from the first residual pass
      // this warp's rows in the residual
      const i64 rb = n * wig / G, re = n * (wig + 1) / G;
      for (int c0 = 0; c0 < nr_all; c0 += kResRhs) {
        const int nr = min(kResRhs, nr_all - c0);
        const double* Bc = Bs + c0 * d.ldb;
        double* Xc = Xs + c0 * d.ldb;
        float* Rc = Rs + (i64)c0 * n;
        double bnorm[kResRhs];
        for (int c = 0; c < kResRhs; ++c) {
          double bn = 0.0;
          if (c < nr)
            for (i64 i = tid; i < n; i += NT) bn = fmax(bn, fabs(Bc[i + c * d.ldb]));
          bnorm[c] = grp_max<G>(bn, red);
        }
        int it = 0;
        double be = 0.0;
        for (;;) {
          double rnorm[kResRhs], xnorm[kResRhs], an = 0.0;
          const bool first = anorm < 0.0;
          residual_rows<Q>(n, rb, re, kl, ku, nr, A + kl, ldab, Bc, Xc, d.ldb, Rc, first, an, rnorm, xnorm);
          if (first) anorm = grp_max<G>(an, red);
          be = 0.0;
          for (int c = 0; c < kResRhs; ++c) {
            const double rn = grp_max<G>(rnorm[c], red), xn = grp_max<G>(xnorm[c], red);
            if (c >= nr) continue;
            const double den = anorm * xn + bnorm[c];
            const double bc = den > 0.0 ? rn / den : rn;
            be = (bc > be || bc != bc) ? bc : be;
          }
          if (!(be > p.tol) || it >= p.maxit) break;  // NaN stops too
          sync();
          solve32(nr, Rc);
          sync();
          for (i64 e = tid; e < n * nr; e += NT) {
            const i64 c = e / n, i = e - c * n;
            Xc[i + c * d.ldb] += (double)Rc[e];
          }
          sync();
          ++it;
        }
        its_max = max(its_max, it);
        berr_max = (be > berr_max || be != be) ? be : berr_max;
      }
    }
    if (tid == 0) {
      p.iters[s] = its_max;
      p.berr[s] = berr_max;
    }
    sync();
  }
}

// Two-part schedule, as gbsv_batched_kernel: wide systems (order[0..n_wide)) one per
// CTA of W warps, then narrow systems one per warp in group_elems-float slices.
template <int W, int Q>
__global__ void __launch_bounds__(32 * W) dsgbsv_batched_kernel(const MixedParams p, i64 n_wide) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* base = reinterpret_cast<float*>(smem_raw);
  int idx;
  for (;;) {
    idx = next_item<W>(p.counter, reinterpret_cast<int*>(base));
    if (idx >= n_wide) break;
    dsgbsv_system<W, Q>(p, p.order ? p.order[idx] : idx, base);
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
    dsgbsv_system<1, Q>(p, p.order ? p.order[my] : my, ws);
    my = -1;
  }
}

// Floats of one group's shared memory for systems up to (kl, ku): FP32 factor window,
// FP32 solve chunk, FP64 residual scratch; 0 when the refined solve does not support
// the band (kl + ku above the residual window).
template <int NLMAX>
static i64 mixed_group_elems(i64 kl, i64 ku) {
  if (kl + ku + 32 > 32 * kResQWide) return 0;
  const i64 fac = gbtrf_smem_elems<4>((int)kl, (int)ku);
  const i64 reg = (reg_group_bytes<float, NLMAX, kMaxRhs>(kl, ku) + 3) / 4;
  const i64 f = std::max(std::max(std::max(fac, gbtrs_smem_elems((int)kl, (int)ku)), (i64)(kHdr + 16)), reg);
  return ((f + 3) / 4) * 4;
}

template <int W, int Q>
static int dsgbsv_launch(MixedParams p, const bm_gb_schedule& sc, cudaStream_t stream, const char* name) {
  const i64 we = sc.n_wide > 0 ? mixed_group_elems<32 * W>(sc.wide_kl, sc.wide_ku) : 1;
  const i64 ne = sc.n_wide < p.count ? mixed_group_elems<32>(sc.narrow_kl, sc.narrow_ku) : 1;
  if (we == 0 || ne == 0) {
    set_error("%s: kl + ku exceeds the refined solve's limit of %d", name, 32 * kResQWide - 32);
    return BM_ERR_UNSUPPORTED;
  }
  p.group_elems = sc.n_wide < p.count ? ne : 0;
  const i64 bytes = std::max(std::max(we, W * (sc.n_wide < p.count ? ne : 0)), (i64)kHdr) * 4;
  if (bytes > 227 * 1024) {
    set_error("%s: the schedule's shared memory (%lld bytes) exceeds the per-CTA limit", name, (long long)bytes);
    return BM_ERR_UNSUPPORTED;
  }
  const void* kfn = (const void*)dsgbsv_batched_kernel<W, Q>;
  int r = cuda_status(ensure_smem(kfn, (int)bytes), name);
  if (r) return r;
  int per_sm = 0;
  r = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dsgbsv_batched_kernel<W, Q>, 32 * W, (int)bytes),
                  name);
  if (r) return r;
  per_sm = std::max(per_sm, 1);
  const i64 need = sc.n_wide + ceil_div(p.count - sc.n_wide, (i64)W);
  const i64 grid = std::min<i64>((i64)num_sms() * per_sm, std::max<i64>(need, 1));
  r = cuda_status(cudaMemsetAsync(p.counter, 0, sizeof(int32_t), stream), name);
  if (r) return r;
  dsgbsv_batched_kernel<W, Q><<<(unsigned)grid, 32 * W, (int)bytes, stream>>>(p, sc.n_wide);
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
  const i64 kvmax = std::max(sc->n_wide > 0 ? sc->wide_kl + sc->wide_ku : 0,
                             sc->n_wide < p.count ? sc->narrow_kl + sc->narrow_ku : 0);
  const bool wideq = kvmax + 32 > 32 * kResQ;
  if (sc->warps == 8) return wideq ? dsgbsv_launch<8, kResQWide>(p, *sc, stream, name)
                                   : dsgbsv_launch<8, kResQ>(p, *sc, stream, name);
  return wideq ? dsgbsv_launch<4, kResQWide>(p, *sc, stream, name) : dsgbsv_launch<4, kResQ>(p, *sc, stream, name);
}

}  // namespace bm

extern "C" int bm_dsgbsv_batched(int64_t count, const bm_gb_desc* descs, const int32_t* order, const double* AB,
                                 const double* B, double* X, int64_t* ipiv, int64_t* info, float* AB32, float* R32,
                                 int32_t* iters, double* berr, int32_t* counter, double tol, int64_t maxit,
                                 int64_t max_kl, int64_t max_ku, bm_stream_t stream) {
  bm::MixedParams p;
  p.count = count; p.descs = descs; p.order = order; p.AB = AB; p.B = B; p.X = X; p.ipiv = ipiv; p.info = info;
  p.AB32 = AB32; p.R32 = R32; p.iters = iters; p.berr = berr; p.counter = counter; p.tol = tol;
  p.maxit = (int)std::min<int64_t>(maxit, 1 << 20);
  p.group_elems = 0;
  if (maxit < 0) return -15;
  if (max_kl < 0) return -17;
  if (max_ku < 0) return -18;
  bm_gb_schedule sc;  // every system wide (4 warps) once the widest window holds 512 entries, else narrow
  sc.n_wide = (max_kl + 1) * (max_kl + max_ku + 1) >= 512 ? count : 0;
  sc.warps = 4;
  sc.wide_kl = sc.narrow_kl = max_kl;
  sc.wide_ku = sc.narrow_ku = max_ku;
  const int r = bm::dsgbsv_batched_impl(p, &sc, reinterpret_cast<cudaStream_t>(stream), "bm_dsgbsv_batched");
  return r == -4 ? -17 : r;
}

extern "C" int bm_dsgbsv_batched_sched(int64_t count, const bm_gb_desc* descs, const int32_t* order,
                                       const bm_gb_schedule* sched, const double* AB, const double* B, double* X,
                                       int64_t* ipiv, int64_t* info, float* AB32, float* R32, int32_t* iters,
                                       double* berr, int32_t* counter, double tol, int64_t maxit, bm_stream_t stream) {
  bm::MixedParams p;
  p.count = count; p.descs = descs; p.order = order; p.AB = AB; p.B = B; p.X = X; p.ipiv = ipiv; p.info = info;
  p.AB32 = AB32; p.R32 = R32; p.iters = iters; p.berr = berr; p.counter = counter; p.tol = tol;
  p.maxit = (int)std::min<int64_t>(maxit, 1 << 20);
  p.group_elems = 0;
  if (maxit < 0) return -16;
  return bm::dsgbsv_batched_impl(p, sched, reinterpret_cast<cudaStream_t>(stream), "bm_dsgbsv_batched_sched");
}
