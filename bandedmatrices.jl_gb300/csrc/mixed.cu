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

// r = b - A x for one system, written to r32 (FP32); returns ||r||_inf (FP64).
// Column-oriented: for each column j, lanes update y[j-ku .. j+kl] (a coalesced read
// of band column j); a sliding window of y in shared memory holds the partial sums.
// Rows are emitted once every column that touches them has been added.
__device__ double residual_warp(i64 n, int kl, int ku, const double* __restrict__ ab, i64 ldab,
                                const double* __restrict__ b, const double* __restrict__ x, float* __restrict__ r32,
                                double* __restrict__ Y, double& xnorm) {
  const int lane = threadIdx.x & 31;
  const int kv = kl + ku;          // ab points at the band: A(i,j) = ab[(ku + i - j) + j*ldab]
  const int W = 32 + kl + ku;      // window: rows j0-ku .. j0+31+kl
  double rnorm = 0.0, xn = 0.0;
  for (int s = lane; s < W; s += 32) Y[s] = 0.0;
  __syncwarp();
  for (i64 j0 = 0; j0 < n; j0 += 32) {
    const int jn = (int)min((i64)32, n - j0);
    // window row index w <-> matrix row j0 - ku + w
    for (int t = 0; t < jn; ++t) {
      const i64 j = j0 + t;
      const double xj = x[j];
      if (lane == 0) xn = fmax(xn, fabs(xj));
      const double* col = ab + j * ldab;  // band column j: matrix rows j-ku .. j+kl
      for (int r = lane; r <= kv; r += 32) {
        const i64 i = j - ku + r;
        if (i >= 0 && i < n) Y[t + r] = fma(col[r], xj, Y[t + r]);
      }
      __syncwarp();
    }
    // rows j0-ku .. j0-ku+jn-1 (window 0..jn-1) are complete when j0+jn == n or
    // all their columns (<= i+ku) were seen: i + ku <= j0 + jn - 1  <=>  w <= jn - 1
    for (int w = lane; w < jn; w += 32) {
      const i64 i = j0 - ku + w;
      if (i >= 0 && i < n) {
        const double ri = b[i] - Y[w];
        r32[i] = (float)ri;
        rnorm = fmax(rnorm, fabs(ri));
      }
    }
    __syncwarp();
    // slide the window by jn
    warp_shift_down(Y, W - jn, jn);
    for (int s = W - jn + lane; s < W; s += 32) Y[s] = 0.0;
    __syncwarp();
  }
  // tail rows n-ku .. n-1 (window 0..ku-1 after the last slide)
  for (int w = lane; w < ku; w += 32) {
    const i64 i = n - ku + w;
    if (i >= 0) {
      const double ri = b[i] - Y[w];
      r32[i] = (float)ri;
      rnorm = fmax(rnorm, fabs(ri));
    }
  }
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    rnorm = fmax(rnorm, __shfl_xor_sync(0xffffffffu, rnorm, off));
    xn = fmax(xn, __shfl_xor_sync(0xffffffffu, xn, off));
  }
  xnorm = xn;
  __syncwarp();
  return rnorm;
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
  float* R32;        // FP32 work vector per system (offsets = ipiv offsets)
  int32_t* iters;    // per system: corrections taken (max over right-hand sides)
  double* berr;      // per system: final backward error (max over right-hand sides)
  int32_t* counter;
  double tol;
  int maxit;
  i64 warp_elems;    // bytes of shared memory per warp / 4
};

__global__ void __launch_bounds__(128) dsgbsv_batched_kernel(const MixedParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float* smem = reinterpret_cast<float*>(smem_raw) + warp * p.warp_elems;
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(p.counter, 1);
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (idx >= p.count) break;
    const int s = p.order ? p.order[idx] : idx;
    const bm_gb_desc d = p.descs[s];
    const int kl = (int)d.kl, ku = (int)d.ku, kv = kl + ku;
    const i64 n = d.n, ldab = d.ldab;
    const double* A = p.AB + d.ab_offset;
    float* A32 = p.AB32 + d.ab_offset;
    i64* ip = p.ipiv + d.ipiv_offset;
    float* r32 = p.R32 + d.ipiv_offset;
    // ---- round to FP32 (top kl rows zero) and ||A||_inf (max row sum of |a_ij|)
    double anorm = 0.0;
    for (i64 i0 = 0; i0 < n; i0 += 32) {
      const i64 i = i0 + lane;
      double rs = 0.0;
      if (i < n)
        for (int dd = -kl; dd <= ku; ++dd) {
          const i64 j = i + dd;
          if (j >= 0 && j < n) rs += fabs(A[(kv + i - j) + j * ldab]);
        }
      anorm = fmax(anorm, rs);
    }
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) anorm = fmax(anorm, __shfl_xor_sync(0xffffffffu, anorm, off));
    const i64 tot = ldab * n;
    for (i64 e = lane; e < tot; e += 32) {
      const i64 r = e % ldab;
      A32[e] = r < kl ? 0.0f : (float)A[e];
    }
    __syncwarp();
    // ---- FP32 factorization
    const i64 inf = gbtrf_warp<float, 4>(n, n, kl, ku, A32, ldab, ip, smem);
    if (lane == 0) p.info[s] = inf;
    int its_max = 0;
    double berr_max = 0.0;
    if (inf == 0) {
      double* Yw = reinterpret_cast<double*>(smem);  // residual window (the factor window is free now)
      for (i64 c = 0; c < d.nrhs; ++c) {
        const double* b = p.B + d.b_offset + c * d.ldb;
        double* x = p.X + d.b_offset + c * d.ldb;
        // x0 = LU32 \ b
        double bnorm = 0.0;
        for (i64 i = lane; i < n; i += 32) {
          r32[i] = (float)b[i];
          bnorm = fmax(bnorm, fabs(b[i]));
        }
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) bnorm = fmax(bnorm, __shfl_xor_sync(0xffffffffu, bnorm, off));
        __syncwarp();
        gbtrs_warp<float>(false, n, kl, ku, A32, ldab, ip, r32, smem);
        __syncwarp();
        for (i64 i = lane; i < n; i += 32) x[i] = (double)r32[i];
        __syncwarp();
        int it = 0;
        double be = 0.0;
        for (;;) {
          double xnorm = 0.0;
          const double rnorm = residual_warp(n, kl, ku, A + kl, ldab, b, x, r32, Yw, xnorm);
          const double den = anorm * xnorm + bnorm;
          be = den > 0.0 ? rnorm / den : rnorm;
          if (!(be > p.tol) || it >= p.maxit) break;  // NaN stops too
          gbtrs_warp<float>(false, n, kl, ku, A32, ldab, ip, r32, smem);
          __syncwarp();
          for (i64 i = lane; i < n; i += 32) x[i] += (double)r32[i];
          __syncwarp();
          ++it;
        }
        its_max = max(its_max, it);
        berr_max = fmax(berr_max, be);
      }
    }
    if (lane == 0) {
      p.iters[s] = its_max;
      p.berr[s] = berr_max;
    }
    __syncwarp();
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
  const i64 f = std::max(gbtrf_smem_elems<4>(kl, ku), gbtrs_smem_elems(kl, ku));
  const i64 rwin = 2 * (32 + kl + ku);  // doubles as floats
  const i64 welems = ((std::max(f, rwin) + 3) / 4) * 4;
  const i64 wbytes = welems * 4;
  if (wbytes > 227 * 1024) {
    set_error("%s: widest band of the batch exceeds the per-warp window limit", name);
    return BM_ERR_UNSUPPORTED;
  }
  p.warp_elems = welems;
  const int wpc = (int)std::max<i64>(1, std::min<i64>(4, (100 * 1024) / wbytes));
  const int smem = (int)(wpc * wbytes);
  int r = cuda_status(ensure_smem((const void*)dsgbsv_batched_kernel, smem), name);
  if (r) return r;
  int per_sm = 0;
  r = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dsgbsv_batched_kernel, 32 * wpc, smem), name);
  if (r) return r;
  per_sm = std::max(per_sm, 1);
  const i64 grid = std::min<i64>((i64)num_sms() * per_sm, ceil_div(p.count, wpc));
  r = cuda_status(cudaMemsetAsync(p.counter, 0, sizeof(int32_t), stream), name);
  if (r) return r;
  dsgbsv_batched_kernel<<<(unsigned)grid, 32 * wpc, smem, stream>>>(p);
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
  p.warp_elems = 0;
  if (maxit < 0) return -15;
  return bm::dsgbsv_batched_impl(p, max_kl, max_ku, reinterpret_cast<cudaStream_t>(stream), "bm_dsgbsv_batched");
}
