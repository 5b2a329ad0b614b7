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
// Structure: a persistent kernel, tiles of TJ consecutive C columns.  Per tile, thread 0
// streams A's columns [j0-Bu, j0+TJ+Bl), B's columns [j0, j0+TJ) and (beta != 0) C's
// columns into a two-slot shared-memory ring with 1-D TMA bulk copies (mbarrier
// completion).  A warp owns one C column at a time; lane r holds C storage rows
// r, r+32, r+64, ... in registers, so B(v,j) is one broadcast shared load per term.
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

// Generic fallback (any alignment, very wide bands): one thread per C entry.
template <typename T>
__global__ void gbmm_simple_kernel(const GbmmParams<T> p) {
  const int crows = p.Cl + p.Cu + 1;
  const i64 total = p.m * (i64)crows;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
    const i64 j = e / crows;
    const int rc = (int)(e - j * crows);
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
