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

namespace bm {

// R = B - A X on rows [rb, re) for up to kResRhs right-hand sides of one system,
// written to R32 (FP32, leading dim n); returns this warp's partial maxima of |r_c|,
// |x_c| (over the columns it read) and, with want_anorm, of the |A| row sums.  Each
// lane owns window rows w = lane + 32q (q < kResQ) in registers; band columns are
// streamed once per 32-column chunk, every lane reading the entry of its own row (a
// coalesced read of the column), so no shared memory and no synchronisation are
// needed.  Row i accumulates its terms in ascending column order.
constexpr int kResRhs = 4;
constexpr int kResQ = 5;  // window rows 32*kResQ >= 32 + kl + ku  (kl + ku <= 128)

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

template <int G>
__global__ void __launch_bounds__(G == 1 ? 128 : 32 * G) dsgbsv_batched_kernel(const MixedParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int NT = Grp<G>::NT;
  const int grp = G == 1 ? (int)(threadIdx.x >> 5) : 0;
  const int tid = Grp<G>::tid(), wig = tid >> 5;
  float* smem = reinterpret_cast<float*>(smem_raw) + grp * p.group_elems;
  int* hdr = reinterpret_cast<int*>(smem);
  double* red = reinterpret_cast<double*>(smem + kHdr);  // reduction scratch (between phases)
  auto sync = [] { Grp<G>::sync(); };
  for (;;) {
    const int idx = next_item<G>(p.counter, hdr);
    if (idx >= p.count) break;
    const int s = p.order ? p.order[idx] : idx;
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
    // ---- FP32 factorization
    const i64 inf = gbtrf_group<float, 4, G>(n, n, kl, ku, A32, ldab, ip, smem);
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
      gbtrs_all<float, G>(false, n, kl, ku, nr_all, A32, ldab, ip, Rs, n, smem);
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
          residual_rows(n, rb, re, kl, ku, nr, A + kl, ldab, Bc, Xc, d.ldb, Rc, first, an, rnorm, xnorm);
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
          gbtrs_all<float, G>(false, n, kl, ku, nr, A32, ldab, ip, Rc, n, smem);
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

static int dsgbsv_batched_impl(const MixedParams& p0, i64 max_kl, i64 max_ku, cudaStream_t stream,
                               const char* name) {
  MixedParams p = p0;
  if (p.count < 0) return -1;
  if (!p.descs && p.count) return -2;
  if (!p.counter) return -14;
  if (!(p.tol >= 0.0)) return -15;
  if (p.maxit < 0) return -16;
  if (max_kl < 0) return -17;
  if (max_ku < 0) return -18;
  if (p.count == 0) return BM_OK;
  const int kl = (int)max_kl, ku = (int)max_ku;
  // per-warp shared memory: FP32 factor window / FP32 solve chunk / FP64 residual window
  const i64 f = std::max(std::max(gbtrf_smem_elems<4>(kl, ku), gbtrs_smem_elems(kl, ku)), (i64)(kHdr + 16));
  if (kl + ku + 32 > 32 * kResQ) {
    set_error("%s: kl + ku = %d exceeds the refined solve's limit of %d", name, kl + ku, 32 * kResQ - 32);
    return BM_ERR_UNSUPPORTED;
  }
  const i64 welems = ((f + 3) / 4) * 4;
  const i64 wbytes = welems * 4;
  if (wbytes > 227 * 1024) {
    set_error("%s: widest band of the batch exceeds the per-warp window limit", name);
    return BM_ERR_UNSUPPORTED;
  }
  p.group_elems = welems;
  const bool cta = (kl + 1) * (kl + ku + 1) >= 512;
  const int gpc = cta ? 1 : (int)std::max<i64>(1, std::min<i64>(4, (100 * 1024) / wbytes));
  const int threads = cta ? 128 : 32 * gpc;
  const int smem = (int)(gpc * wbytes);
  const void* kfn = cta ? (const void*)dsgbsv_batched_kernel<4> : (const void*)dsgbsv_batched_kernel<1>;
  int r = cuda_status(ensure_smem(kfn, smem), name);
  if (r) return r;
  int per_sm = 0;
  r = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, threads, smem), name);
  if (r) return r;
  per_sm = std::max(per_sm, 1);
  const i64 grid = std::min<i64>((i64)num_sms() * per_sm, ceil_div(p.count, gpc));
  r = cuda_status(cudaMemsetAsync(p.counter, 0, sizeof(int32_t), stream), name);
  if (r) return r;
  if (cta)
    dsgbsv_batched_kernel<4><<<(unsigned)grid, threads, smem, stream>>>(p);
  else
    dsgbsv_batched_kernel<1><<<(unsigned)grid, threads, smem, stream>>>(p);
  return launch_status(name);
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
  return bm::dsgbsv_batched_impl(p, max_kl, max_ku, reinterpret_cast<cudaStream_t>(stream), "bm_dsgbsv_batched");
}
