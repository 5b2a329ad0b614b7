// gbmv: y <- alpha*op(A)*x + beta*y on LAPACK band storage.
//
// Replaces the xGBMV ccall of BandedMatrices.jl (src/blas.jl:16-28; stdlib
// BLAS.gbmv! from banded_gbmv!, src/generic/matmul.jl:21-23).
//
// Fast path (incx = incy = 1, 16-byte aligned A and x): a persistent kernel,
// one or two CTAs per SM.  Work is cut into tiles of consecutive outputs; for each
// tile a producer warp streams the band columns the tile touches, and the x window,
// from HBM into a shared-memory ring of `stages` buffers with 1-D TMA bulk copies
// (cp.async.bulk, completion on an mbarrier), while 15 consumer warps reduce earlier
// buffers and hand each one back through an mbarrier of its own.  Each output element is owned by one thread and accumulated
// in the reference-BLAS order (see below), so the result is deterministic and
// equal, bit for bit, to reference dgbmv compiled with fused multiply-adds.
//
//   'N': y_i = beta*y_i, then y_i = fma(alpha*x_j, A(i,j), y_i) for j ascending
//        (the column-oriented loop of reference DGBMV);
//   'T': t = sum_i A(i,j)*x_i accumulated with fma for i ascending,
//        y_j = fma(alpha, t, beta*y_j).
//
// Roofline: HBM.  Algorithmic bytes per call = s*(lda*n + |x| + |y|*(beta!=0 ? 2 : 1)).
#include <cstdio>
#include <cstdlib>

#include "common.cuh"

namespace bm {

template <typename T>
struct GbmvParams {
  i64 m, n, kl, ku, lda;
  T alpha, beta;
  const T* A;
  const T* x;
  T* y;
  i64 tile;    // outputs per tile
  i64 ntiles;
  int stages;
  uint32_t stage_bytes;  // bytes per ring slot (A part + x part), multiple of 128
  uint32_t xoff;         // byte offset of the x part inside a slot
  int* status;
  const int* skip;       // device flag: nonzero -> the launch does nothing (NULL: always run)
};

template <typename T>
struct Region {
  i64 gs;      // first element held in smem (rounded down to 16 bytes)
  i64 ge;      // end of the bulk-copied part (rounded down to 16 bytes)
  i64 end;     // one past the last element needed
};

template <typename T>
__device__ __forceinline__ Region<T> make_region(i64 start, i64 end) {
  constexpr i64 q = 16 / sizeof(T);
  Region<T> r;
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

// Column range of A and element range of x touched by tile t.
template <typename T, bool TRANS>
__device__ __forceinline__ void tile_ranges(const GbmvParams<T>& p, i64 t, i64& o0, i64& o1, i64& c0,
                                            i64& c1, i64& x0, i64& x1) {
  o0 = t * p.tile;
  o1 = min(o0 + p.tile, TRANS ? p.n : p.m);
  if (!TRANS) {
    c0 = max((i64)0, o0 - p.kl);
    c1 = min(p.n, o1 + p.ku);
    if (c1 < c0) c1 = c0;
    x0 = c0;
    x1 = c1;
  } else {
    c0 = o0;
    c1 = o1;
    x0 = max((i64)0, o0 - p.ku);
    x1 = min(p.m, o1 + p.kl);
    if (x1 < x0) x1 = x0;
  }
}

// Ring protocol (no block-wide barrier in the loop).  Warp 0 is the producer, warps
// 1..15 the consumers.  Slot s has three mbarriers:
//   full[s]  (2 arrivals + tx bytes): the producer's arrive.expect_tx before the bulk
//            copies, and its arrive after it stored the ragged tails;
//   ready[s] (1 arrival, alpha != 1 in 'N' only): the producer scaled x by alpha;
//   empty[s] (15 arrivals): each consumer warp is done reading the slot.
// Every wait is bounded (kSpinLimit polls); on expiry the status word gets
// BM_STATUS_TIMEOUT, the consumers stop and the producer waits (bounded) for the
// copies still in flight before the CTA exits.
constexpr int kGbmvThreads = 512;
constexpr int kGbmvConsumers = kGbmvThreads / 32 - 1;

template <typename T, bool TRANS>
__device__ __forceinline__ bool produce_tile(const GbmvParams<T>& p, unsigned char* slots, uint64_t* full,
                                             uint64_t* ready, i64 k, int lane) {
  const i64 t = (i64)blockIdx.x + k * (i64)gridDim.x;
  const int s = (int)(k % p.stages);
  i64 o0, o1, c0, c1, x0, x1;
  tile_ranges<T, TRANS>(p, t, o0, o1, c0, c1, x0, x1);
  const Region<T> ra = make_region<T>(c0 * p.lda, c1 * p.lda);
  const Region<T> rx = make_region<T>(x0, x1);
  T* sa = reinterpret_cast<T*>(slots + (size_t)s * p.stage_bytes);
  T* sx = reinterpret_cast<T*>(slots + (size_t)s * p.stage_bytes + p.xoff);
  if (lane == 0) {
    const uint32_t ba = (uint32_t)((ra.ge - ra.gs) * (i64)sizeof(T));
    const uint32_t bx = (uint32_t)((rx.ge - rx.gs) * (i64)sizeof(T));
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&full[s], ba + bx);
    if (ba) bulk_g2s(sa, p.A + ra.gs, ba, &full[s]);
    if (bx) bulk_g2s(sx, p.x + rx.gs, bx, &full[s]);
  }
  // ragged tails (< 16 bytes) the bulk copies leave out
  const int na = (int)(ra.end - ra.ge), nx = (int)(rx.end - rx.ge);
  if (lane < na) sa[ra.ge - ra.gs + lane] = p.A[ra.ge + lane];
  else if (lane >= 16 && lane - 16 < nx) sx[rx.ge - rx.gs + lane - 16] = p.x[rx.ge + lane - 16];
  __syncwarp();
  if (lane == 0) mbar_arrive(&full[s]);
  if (!TRANS && p.alpha != T(1)) {  // x <- alpha*x once per slot (the column dgbmv's temp)
    const bool ok = mbar_wait(&full[s], (uint32_t)((k / p.stages) & 1));
    if (!__all_sync(0xffffffffu, ok)) return false;
    for (i64 e = x0 + lane; e < x1; e += 32) sx[e - rx.gs] = p.alpha * sx[e - rx.gs];
    __syncwarp();
    if (lane == 0) mbar_arrive(&ready[s]);
  }
  return true;
}

template <typename T, bool TRANS>
__global__ void __launch_bounds__(kGbmvThreads) gbmv_tma_kernel(const GbmvParams<T> p) {
  if (p.skip && *reinterpret_cast<volatile const int*>(p.skip)) return;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* ready = full + 8;
  uint64_t* empty = full + 16;
  unsigned char* slots = smem + 256;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < p.stages; ++s) {
      mbar_init(&full[s], 2);
      mbar_init(&ready[s], 1);
      mbar_init(&empty[s], kGbmvConsumers);
    }
    fence_mbar_init();
  }
  __syncthreads();
  const i64 my_tiles = p.ntiles > blockIdx.x ? (p.ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;

  if (warp == 0) {  // ---------------------------------------------------------- producer
    bool ok = true;
    i64 k = 0;
    for (; k < my_tiles; ++k) {
      if (k >= p.stages) {  // the consumers released tile k - stages from this slot
        const bool w = mbar_wait(&empty[k % p.stages], (uint32_t)((k / p.stages - 1) & 1));
        ok = __all_sync(0xffffffffu, w);
        if (!ok) break;
      }
      if (!produce_tile<T, TRANS>(p, slots, full, ready, k, lane)) {
        ok = false;
        ++k;
        break;
      }
    }
    if (!ok) {
      if (lane == 0) record_status(p.status, BM_STATUS_TIMEOUT);
    }
    // let every copy this CTA issued land before it exits
    for (i64 kk = std::max<i64>((i64)0, k - p.stages); kk < k; ++kk)
      (void)mbar_wait(&full[kk % p.stages], (uint32_t)((kk / p.stages) & 1));
    return;
  }

  // ------------------------------------------------------------------------ consumers
  const int ct = threadIdx.x - 32, bd = kGbmvThreads - 32;
  // The tests of beta once, on the integer side: an FP64 comparison per output would
  // occupy GB300's slow FP64 pipe, which the Float64 products already saturate.
  const bool beta0 = p.beta == T(0);
  for (i64 k = 0; k < my_tiles; ++k) {
    const i64 t = (i64)blockIdx.x + k * (i64)gridDim.x;
    const int s = (int)(k % p.stages);
    const uint32_t phase = (uint32_t)((k / p.stages) & 1);
    bool ok = mbar_wait(&full[s], phase);
    if (ok && !TRANS && p.alpha != T(1)) ok = mbar_wait(&ready[s], phase);
    if (!__all_sync(0xffffffffu, ok)) {
      if (lane == 0) record_status(p.status, BM_STATUS_TIMEOUT);
      return;
    }
    i64 o0, o1, c0, c1, x0, x1;
    tile_ranges<T, TRANS>(p, t, o0, o1, c0, c1, x0, x1);
    const Region<T> ra = make_region<T>(c0 * p.lda, c1 * p.lda);
    const Region<T> rx = make_region<T>(x0, x1);
    const T* sa = reinterpret_cast<const T*>(slots + (size_t)s * p.stage_bytes);
    const T* sx = reinterpret_cast<const T*>(slots + (size_t)s * p.stage_bytes + p.xoff);

    // Tile-local 32-bit indexing.  For 'N', outputs are rows i and A's columns are
    // local to c0; for 'T', outputs are columns j and x's rows are local to x0.
    const int nout = (int)(o1 - o0);
    const int lda = (int)p.lda, kl = (int)p.kl, ku = (int)p.ku, kb = kl + ku + 1;
    if (!TRANS) {
      const int abase = (int)(c0 * p.lda - ra.gs) + ku;  // + jj*(lda-1) + li
      const int xbase = (int)(c0 - rx.gs);               // + jj
      const i64 nmax = p.n - 1 - c0;                     // last local column
      const int off = (int)(o0 - c0);                    // local index of row o0
      for (int tt = ct; tt < nout; tt += 2 * bd) {
        const int t2 = tt + bd;
        const int li = off + tt, li2 = off + t2;
        const bool two = t2 < nout;
        const bool full1 = (o0 + tt - kl >= 0) && (li + ku <= nmax);
        const bool full2 = two && (o0 + t2 - kl >= 0) && (li2 + ku <= nmax);
        T acc1 = beta0 ? T(0) : p.beta * p.y[o0 + tt];
        T acc2 = (two && !beta0) ? p.beta * p.y[o0 + t2] : T(0);
        if (full1 && full2) {
          // two independent chains over all kb terms
          int ia = abase + (li - kl) * (lda - 1) + li, ix = xbase + li - kl;
          int ia2 = ia + bd * lda, ix2 = ix + bd;
#pragma unroll 4
          for (int q = 0; q < kb; ++q) {
            acc1 = fma(sx[ix], sa[ia], acc1);
            acc2 = fma(sx[ix2], sa[ia2], acc2);
            ia += lda - 1; ia2 += lda - 1; ++ix; ++ix2;
          }
        } else {
          {
            const int jlo = (int)max((i64)(li - kl), -c0), jhi = (int)min((i64)(li + ku), nmax);
            int ia = abase + jlo * (lda - 1) + li, ix = xbase + jlo;
            for (int jj = jlo; jj <= jhi; ++jj) {
              acc1 = fma(sx[ix], sa[ia], acc1);
              ia += lda - 1; ++ix;
            }
          }
          if (two) {
            const int jlo = (int)max((i64)(li2 - kl), -c0), jhi = (int)min((i64)(li2 + ku), nmax);
            int ia = abase + jlo * (lda - 1) + li2, ix = xbase + jlo;
            for (int jj = jlo; jj <= jhi; ++jj) {
              acc2 = fma(sx[ix], sa[ia], acc2);
              ia += lda - 1; ++ix;
            }
          }
        }
        p.y[o0 + tt] = acc1;
        if (two) p.y[o0 + t2] = acc2;
      }
    } else {
      const int abase = (int)(o0 * p.lda - ra.gs) + ku;  // + lj*lda + (li - lj) with li local to o0
      const int xbase = (int)(o0 - rx.gs);               // + li
      const i64 mmax = p.m - 1 - o0;
      for (int tt = ct; tt < nout; tt += 2 * bd) {
        const int t2 = tt + bd;
        const bool two = t2 < nout;
        const bool full1 = (o0 + tt - ku >= 0) && (tt + kl <= mmax);
        const bool full2 = two && (o0 + t2 - ku >= 0) && (t2 + kl <= mmax);
        T acc1 = T(0), acc2 = T(0);
        if (full1 && full2) {
          int ia = abase + tt * lda - ku, ix = xbase + tt - ku;
          int ia2 = ia + bd * lda, ix2 = ix + bd;
#pragma unroll 4
          for (int q = 0; q < kb; ++q) {
            acc1 = fma(sa[ia], sx[ix], acc1);
            acc2 = fma(sa[ia2], sx[ix2], acc2);
            ++ia; ++ia2; ++ix; ++ix2;
          }
        } else {
          {
            const int ilo = (int)max((i64)(tt - ku), -o0), ihi = (int)min((i64)(tt + kl), mmax);
            int ia = abase + tt * lda + ilo - tt, ix = xbase + ilo;
            for (int li = ilo; li <= ihi; ++li) {
              acc1 = fma(sa[ia], sx[ix], acc1);
              ++ia; ++ix;
            }
          }
          if (two) {
            const int ilo = (int)max((i64)(t2 - ku), -o0), ihi = (int)min((i64)(t2 + kl), mmax);
            int ia = abase + t2 * lda + ilo - t2, ix = xbase + ilo;
            for (int li = ilo; li <= ihi; ++li) {
              acc2 = fma(sa[ia], sx[ix], acc2);
              ++ia; ++ix;
            }
          }
        }
        const T y1 = beta0 ? T(0) : p.beta * p.y[o0 + tt];
        p.y[o0 + tt] = fma(p.alpha, acc1, y1);
        if (two) {
          const T y2 = beta0 ? T(0) : p.beta * p.y[o0 + t2];
          p.y[o0 + t2] = fma(p.alpha, acc2, y2);
        }
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
}

// Any strides: one thread per output element, same accumulation order.
template <typename T, bool TRANS>
__global__ void gbmv_strided_kernel(i64 m, i64 n, i64 kl, i64 ku, T alpha, const T* __restrict__ A, i64 lda,
                                    const T* __restrict__ x, i64 incx, T beta, T* __restrict__ y, i64 incy,
                                    const int* skip) {
  if (skip && *reinterpret_cast<volatile const int*>(skip)) return;
  const i64 leny = TRANS ? n : m, lenx = TRANS ? m : n;
  const i64 kx = incx > 0 ? 0 : -(lenx - 1) * incx;
  const i64 ky = incy > 0 ? 0 : -(leny - 1) * incy;
  for (i64 o = (i64)blockIdx.x * blockDim.x + threadIdx.x; o < leny; o += (i64)gridDim.x * blockDim.x) {
    T* yp = y + ky + o * incy;
    if (!TRANS) {
      const i64 i = o;
      const i64 jlo = max((i64)0, i - kl), jhi = min(n - 1, i + ku);
      T acc = (beta == T(0)) ? T(0) : beta * *yp;
      if (alpha != T(0))
        for (i64 j = jlo; j <= jhi; ++j) acc = fma(alpha * x[kx + j * incx], A[j * lda + ku + i - j], acc);
      *yp = acc;
    } else {
      const i64 j = o;
      const i64 ilo = max((i64)0, j - ku), ihi = min(m - 1, j + kl);
      T acc = T(0);
      for (i64 i = ilo; i <= ihi; ++i) acc = fma(A[j * lda + ku + i - j], x[kx + i * incx], acc);
      const T y0 = (beta == T(0)) ? T(0) : beta * *yp;
      *yp = (alpha == T(0)) ? y0 : fma(alpha, acc, y0);
    }
  }
}

// skip: optional device flag read by the kernels at launch (nonzero: no work), so a
// caller can enqueue the call ahead of a device-side decision.
template <typename T>
static int gbmv_impl(char trans, i64 m, i64 n, i64 kl, i64 ku, T alpha, const T* A, i64 lda, const T* x, i64 incx,
                     T beta, T* y, i64 incy, cudaStream_t stream, const char* name, const int* skip = nullptr) {
  const bool notr = (trans == 'N' || trans == 'n');
  if (!notr && !(trans == 'T' || trans == 't' || trans == 'C' || trans == 'c')) return -1;
  if (m < 0) return -2;
  if (n < 0) return -3;
  if (kl < 0) return -4;
  if (ku < 0) return -5;
  if (lda < kl + ku + 1) return -8;
  if (incx == 0) return -10;
  if (incy == 0) return -13;
  if (m == 0 || n == 0 || (alpha == T(0) && beta == T(1))) return BM_OK;
  const i64 leny = notr ? m : n;
  const int nsm = num_sms();

  const bool aligned = ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(x)) & 15) == 0;
  const i64 s = sizeof(T);
  const i64 halo = kl + ku;
  const i64 per_out = (lda + 1) * s;  // bytes of A plus x per band column

  // Tile selection: a ring of `stages` slots per CTA, `ctas` CTAs per SM.
  // BM_GBMV_CFG="ctas,stages,kbytes_per_cta" overrides the search (tuning).
  int ctas = 1, stages = 0;
  i64 tile = 0, budget = 220 * 1024;
  if (const char* env = getenv("BM_GBMV_CFG")) {
    int c = 0, st = 0, kb = 0;
    if (sscanf(env, "%d,%d,%d", &c, &st, &kb) == 3 && c >= 1 && c <= 2 && st >= 2 && st <= 8 && kb >= 16 &&
        kb <= 224) {
      ctas = c;
      stages = st;
      budget = (i64)kb * 1024;
    }
  }
  auto tile_for = [&](int st) {
    const i64 slot = budget / st;
    const i64 cols = (slot - 512) / per_out;
    return notr ? cols - halo : cols - (halo * s + per_out - 1) / per_out;
  };
  if (!stages) {
    // Measured on GB300 (n = 2^24, l = u in {1, 8, 32}, f32 and f64): for 'N' one CTA
    // per SM with two large ring slots (three for tridiagonal bands) is best or within
    // 4% of best; 'T' gains from two CTAs per SM when the band is narrow.
    stages = (notr && halo <= 2) ? 3 : 2;
    if (!notr && halo <= 16) {
      ctas = 2;
      budget = 110 * 1024;
    }
  }
  tile = tile_for(stages);
  tile = std::min<i64>(tile, 8192);
  const i64 want = ceil_div(leny, (i64)nsm * ctas * 2);  // >= ~2 tiles per CTA on small problems
  if (want < tile) tile = std::min<i64>(tile, std::max<i64>(64, ((want + 63) / 64) * 64));

  if (incx != 1 || incy != 1 || !aligned || alpha == T(0) || tile < 32 || (lda * n) >= ((i64)1 << 40)) {
    // Generic path: any strides / alignment, or a band too wide for a staged tile.
    const int threads = 256;
    const i64 blocks = std::min<i64>(ceil_div(leny, threads), (i64)nsm * 32);
    if (notr)
      gbmv_strided_kernel<T, false><<<(unsigned)blocks, threads, 0, stream>>>(m, n, kl, ku, alpha, A, lda, x, incx,
                                                                              beta, y, incy, skip);
    else
      gbmv_strided_kernel<T, true><<<(unsigned)blocks, threads, 0, stream>>>(m, n, kl, ku, alpha, A, lda, x, incx,
                                                                             beta, y, incy, skip);
    return launch_status(name);
  }

  GbmvParams<T> p;
  p.m = m; p.n = n; p.kl = kl; p.ku = ku; p.lda = lda;
  p.alpha = alpha; p.beta = beta; p.A = A; p.x = x; p.y = y;
  p.tile = tile;
  p.ntiles = ceil_div(leny, tile);
  p.stages = stages;
  const i64 cols = notr ? tile + halo : tile;
  const i64 xlen = tile + halo;
  const i64 abytes = ((cols * lda + 2 * (16 / s)) * s + 127) / 128 * 128;
  const i64 xbytes = ((xlen + 2 * (16 / s)) * s + 127) / 128 * 128;
  p.xoff = (uint32_t)abytes;
  p.stage_bytes = (uint32_t)(abytes + xbytes);
  p.status = status_word();
  p.skip = skip;
  const int smem = 256 + stages * (int)p.stage_bytes;
  if (smem > 227 * 1024) {
    set_error("%s: internal tile selection exceeded shared memory (%d bytes)", name, smem);
    return BM_ERR_UNSUPPORTED;
  }
  const void* kfn = notr ? (const void*)gbmv_tma_kernel<T, false> : (const void*)gbmv_tma_kernel<T, true>;
  int r = cuda_status(ensure_smem(kfn, smem), name);
  if (r) return r;
  const i64 grid = std::min<i64>(p.ntiles, (i64)nsm * ctas);
  if (notr)
    gbmv_tma_kernel<T, false><<<(unsigned)grid, kGbmvThreads, smem, stream>>>(p);
  else
    gbmv_tma_kernel<T, true><<<(unsigned)grid, kGbmvThreads, smem, stream>>>(p);
  return launch_status(name);
}

// Several gbmv products in one launch: vector v (blockIdx.y, grid-stride) computes
// y_v = alpha op(A) x_v + beta y_v with x_v = x + v*xs (stride incx), y_v = y + v*ys
// (stride incy), one thread per output in the order of gbmv_strided_kernel.  This is
// banded x dense ('N', a column of B per vector) and dense x banded ('T', a row of D
// per vector) -- the column / row loops of src/generic/matmul.jl:243-271.
template <typename T, bool TRANS>
__global__ void gbmv_multi_kernel(i64 m, i64 n, i64 kl, i64 ku, i64 nvec, T alpha, const T* __restrict__ A, i64 lda,
                                  const T* __restrict__ x, i64 xs, i64 incx, T beta, T* __restrict__ y, i64 ys,
                                  i64 incy) {
  const i64 leny = TRANS ? n : m;
  for (i64 v = blockIdx.y; v < nvec; v += gridDim.y) {
    const T* xv = x + v * xs;
    T* yv = y + v * ys;
    for (i64 o = (i64)blockIdx.x * blockDim.x + threadIdx.x; o < leny; o += (i64)gridDim.x * blockDim.x) {
      T* yp = yv + o * incy;
      if (!TRANS) {
        const i64 i = o;
        const i64 jlo = max((i64)0, i - kl), jhi = min(n - 1, i + ku);
        T acc = (beta == T(0)) ? T(0) : beta * *yp;
        if (alpha != T(0))
          for (i64 j = jlo; j <= jhi; ++j) acc = fma(alpha * xv[j * incx], A[j * lda + ku + i - j], acc);
        *yp = acc;
      } else {
        const i64 j = o;
        const i64 ilo = max((i64)0, j - ku), ihi = min(m - 1, j + kl);
        T acc = T(0);
        for (i64 i = ilo; i <= ihi; ++i) acc = fma(A[j * lda + ku + i - j], xv[i * incx], acc);
        const T y0 = (beta == T(0)) ? T(0) : beta * *yp;
        *yp = (alpha == T(0)) ? y0 : fma(alpha, acc, y0);
      }
    }
  }
}

// C <- alpha A B + beta C: banded A (m x n), dense B (n x k, ldb), C (m x k, ldc).
template <typename T>
static int gbmm_bd_impl(i64 m, i64 n, i64 kl, i64 ku, i64 k, T alpha, const T* A, i64 lda, const T* B, i64 ldb,
                        T beta, T* C, i64 ldc, cudaStream_t stream, const char* name) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (kl < 0) return -3;
  if (ku < 0) return -4;
  if (k < 0) return -5;
  if (lda < kl + ku + 1) return -8;
  if (ldb < std::max<i64>(1, n)) return -10;
  if (ldc < std::max<i64>(1, m)) return -13;
  if (m == 0 || k == 0 || (alpha == T(0) && beta == T(1))) return BM_OK;
  const int threads = 256;
  const i64 bx = std::min<i64>(ceil_div(m, threads), (i64)num_sms() * 8);
  const i64 by = std::min<i64>(k, 65535);
  gbmv_multi_kernel<T, false><<<dim3((unsigned)bx, (unsigned)by), threads, 0, stream>>>(
      m, n, kl, ku, k, alpha, A, lda, B, ldb, 1, beta, C, ldc, 1);
  return launch_status(name);
}

// C <- alpha D A + beta C: dense D (k x m, ldd), banded A (m x n), C (k x n, ldc).
template <typename T>
static int gbmm_db_impl(i64 m, i64 n, i64 kl, i64 ku, i64 k, T alpha, const T* D, i64 ldd, const T* A, i64 lda,
                        T beta, T* C, i64 ldc, cudaStream_t stream, const char* name) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (kl < 0) return -3;
  if (ku < 0) return -4;
  if (k < 0) return -5;
  if (ldd < std::max<i64>(1, k)) return -8;
  if (lda < kl + ku + 1) return -10;
  if (ldc < std::max<i64>(1, k)) return -13;
  if (n == 0 || k == 0 || (alpha == T(0) && beta == T(1))) return BM_OK;
  const int threads = 256;
  const i64 bx = std::min<i64>(ceil_div(n, threads), (i64)num_sms() * 8);
  const i64 by = std::min<i64>(k, 65535);
  gbmv_multi_kernel<T, true><<<dim3((unsigned)bx, (unsigned)by), threads, 0, stream>>>(
      m, n, kl, ku, k, alpha, A, lda, D, 1, ldd, beta, C, 1, ldc);
  return launch_status(name);
}

// Float64 gbmv with a skip flag, for the other translation units of the library.
int dgbmv_flagged(char trans, i64 m, i64 n, i64 kl, i64 ku, double alpha, const double* A, i64 lda, const double* x,
                  i64 incx, double beta, double* y, i64 incy, const int* skip, cudaStream_t stream, const char* name) {
  return gbmv_impl<double>(trans, m, n, kl, ku, alpha, A, lda, x, incx, beta, y, incy, stream, name, skip);
}

}  // namespace bm

extern "C" int bm_dgbmv(char trans, int64_t m, int64_t n, int64_t kl, int64_t ku, double alpha, const double* A,
                        int64_t lda, const double* x, int64_t incx, double beta, double* y, int64_t incy,
                        bm_stream_t stream) {
  return bm::gbmv_impl<double>(trans, m, n, kl, ku, alpha, A, lda, x, incx, beta, y, incy,
                               reinterpret_cast<cudaStream_t>(stream), "bm_dgbmv");
}

extern "C" int bm_sgbmv(char trans, int64_t m, int64_t n, int64_t kl, int64_t ku, float alpha, const float* A,
                        int64_t lda, const float* x, int64_t incx, float beta, float* y, int64_t incy,
                        bm_stream_t stream) {
  return bm::gbmv_impl<float>(trans, m, n, kl, ku, alpha, A, lda, x, incx, beta, y, incy,
                              reinterpret_cast<cudaStream_t>(stream), "bm_sgbmv");
}

extern "C" int bm_dgbmm_bd(int64_t m, int64_t n, int64_t kl, int64_t ku, int64_t k, double alpha, const double* A,
                           int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                           bm_stream_t stream) {
  return bm::gbmm_bd_impl<double>(m, n, kl, ku, k, alpha, A, lda, B, ldb, beta, C, ldc,
                                  reinterpret_cast<cudaStream_t>(stream), "bm_dgbmm_bd");
}
extern "C" int bm_sgbmm_bd(int64_t m, int64_t n, int64_t kl, int64_t ku, int64_t k, float alpha, const float* A,
                           int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc,
                           bm_stream_t stream) {
  return bm::gbmm_bd_impl<float>(m, n, kl, ku, k, alpha, A, lda, B, ldb, beta, C, ldc,
                                 reinterpret_cast<cudaStream_t>(stream), "bm_sgbmm_bd");
}
extern "C" int bm_dgbmm_db(int64_t m, int64_t n, int64_t kl, int64_t ku, int64_t k, double alpha, const double* D,
                           int64_t ldd, const double* A, int64_t lda, double beta, double* C, int64_t ldc,
                           bm_stream_t stream) {
  return bm::gbmm_db_impl<double>(m, n, kl, ku, k, alpha, D, ldd, A, lda, beta, C, ldc,
                                  reinterpret_cast<cudaStream_t>(stream), "bm_dgbmm_db");
}
extern "C" int bm_sgbmm_db(int64_t m, int64_t n, int64_t kl, int64_t ku, int64_t k, float alpha, const float* D,
                           int64_t ldd, const float* A, int64_t lda, float beta, float* C, int64_t ldc,
                           bm_stream_t stream) {
  return bm::gbmm_db_impl<float>(m, n, kl, ku, k, alpha, D, ldd, A, lda, beta, C, ldc,
                                 reinterpret_cast<cudaStream_t>(stream), "bm_sgbmm_db");
}
