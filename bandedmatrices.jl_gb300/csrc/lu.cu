// Banded LU entry points: xGBTRF / xGBTRS for one system and the batched
// persistent factor+solve.  The device algorithms are in lu.cuh.
//
// Replaces LAPACK.gbtrf! (lu!, src/banded/BandedLU.jl:90-103) and LAPACK.gbtrs!
// (ldiv!, src/banded/linalg.jl:24-30 'N', :41-47 'T').
#include <mutex>

#include "lu.cuh"
#include "lureg.cuh"

namespace bm {

constexpr int kP = 4;  // rows staged ahead by cp.async in gbtrf

template <typename T, int G>
__global__ void __launch_bounds__(32 * G) gbtrf_one_kernel(i64 m, i64 n, int kl, int ku, T* ab, i64 ldab, i64* ipiv,
                                                           i64* info) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const i64 r = gbtrf_group<T, kP, G>(m, n, kl, ku, ab, ldab, ipiv, reinterpret_cast<T*>(smem_raw));
  if (threadIdx.x == 0) *info = r;
}

template <typename T, int G>
__global__ void __launch_bounds__(32 * G) gbtrf_blocked_one_kernel(i64 m, i64 n, int kl, int ku, T* ab, i64 ldab,
                                                                   i64* ipiv, i64* info) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const i64 r = gbtrf_blocked_group<T, G>(m, n, kl, ku, ab, ldab, ipiv, reinterpret_cast<T*>(smem_raw));
  if (threadIdx.x == 0) *info = r;
}

template <typename T, int G>
__global__ void __launch_bounds__(32 * G) gbtrs_one_kernel(bool trans, i64 n, int kl, int ku, i64 nrhs, const T* ab,
                                                           i64 ldab, const i64* ipiv, T* B, i64 ldb, int ch) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // block r sweeps right-hand sides [r*kMaxRhs, (r+1)*kMaxRhs)
  for (i64 r = blockIdx.x; r * kMaxRhs < nrhs; r += gridDim.x)
    gbtrs_all<T, G>(trans, n, kl, ku, min((i64)kMaxRhs, nrhs - r * kMaxRhs), ab, ldab, ipiv, B + r * kMaxRhs * ldb,
                    ldb, reinterpret_cast<T*>(smem_raw), ch);
}

// ------------------------------------------------------------------ wide bands
// Bands whose one-column window does not fit one CTA's shared memory (e.g. kl = ku =
// 512 in Float64): the factorization runs panel by panel over the gbtrf storage in
// global memory, as two launches per panel of kNB columns.
//   * gbtrf_panel_kernel (one CTA): loads the panel -- rows j0 .. j0+kl+kNB-1 of its
//     kNB columns -- into shared memory, takes dgbtf2's steps on it (pivot search,
//     interchange within the panel's columns from the step's own column on, scaling,
//     rank-1 update of the panel's later columns), stores it back (L in dgbtf2's
//     format) with the pivots;
//   * gbtrf_replay_kernel (one warp per column): every column the panel's steps can
//     reach (up to kl+ku to its right) replays the steps in order -- interchange, then
//     the update from the stored multipliers -- on its rows j0 .. j0+kl+kNB-1, kept in
//     the warp's shared memory; the multipliers are staged once per CTA, and a step's
//     interchange and zero-pivot flag come from ipiv and the stored U(j,j).
// Each element therefore receives dgbtf2's sequence of operations: factors and pivots
// equal the unblocked result bit for bit.
constexpr int kWideWarps = 8;

// the top kl rows of gbtrf storage (fill-in) start at zero, as dgbtrf sets them
template <typename T>
__global__ void zero_fill_kernel(i64 n, int kl, T* ab, i64 ldab) {
  const i64 total = n * (i64)kl;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
    const i64 c = e / kl;
    ab[(e - c * kl) + c * ldab] = T(0);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) gbtrf_panel_kernel(i64 m, i64 n, int kl, int ku, i64 j0, T* ab, i64 ldab,
                                                          i64* ipiv, i64* info) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int NT = 256, NB = kNB;
  const int tid = threadIdx.x, lane = tid & 31, wig = tid >> 5;
  const int kv = kl + ku, R = kl + NB, RS = R | 1;
  const i64 mn = min(m, n);
  const int jb = (int)min((i64)NB, mn - j0);
  T* P = reinterpret_cast<T*>(smem_raw);  // panel: column c (0..jb-1) x row r (matrix row j0 + r)
  int* hdr = reinterpret_cast<int*>(P + (i64)RS * NB);  // [0] pivot, [4..] per-warp keys and indices
  // entry (row j0+r, column j0+c) of the storage when it lies in it
  auto sidx = [&](int r, int c) -> i64 {
    const i64 i = j0 + r, col = j0 + c;
    const i64 d = i - col;
    return (i < m && d >= -kv && d <= kl) ? (kv + d) + col * ldab : (i64)-1;
  };
  for (int e = tid; e < R * jb; e += NT) {
    const int c = e / R, r = e - c * R;
    const i64 g = sidx(r, c);
    P[c * RS + r] = g >= 0 ? ab[g] : T(0);
  }
  __syncthreads();
  i64 inf = *info;
  for (int c = 0; c < jb; ++c) {
    const i64 gj = j0 + c;
    const int km = (int)min((i64)kl, m - 1 - gj);
    T* colc = P + c * RS;
    {  // idamax over rows c..c+km: every warp scans rows r = tid, tid+NT, ..., then the
       // warps' (key, first index) pairs are combined (larger key, else smaller index)
      unsigned long long key = 0ull;
      int idx = 0x7fffffff;
      for (int r = tid; r <= km; r += NT) {
        const unsigned long long k = pivot_key(colc[c + r], r == 0);
        if (idx == 0x7fffffff || k > key) {
          key = k;
          idx = r;
        }
      }
      const unsigned hi = (unsigned)(key >> 32), lo = (unsigned)key;
      const unsigned mhi = __reduce_max_sync(0xffffffffu, hi);
      const unsigned mlo = __reduce_max_sync(0xffffffffu, hi == mhi ? lo : 0u);
      const int widx = (int)__reduce_min_sync(0xffffffffu, (hi == mhi && lo == mlo) ? (unsigned)idx : 0x7fffffffu);
      unsigned long long* wk = reinterpret_cast<unsigned long long*>(hdr + 4);  // 8 keys
      int* wi = hdr + 4 + 2 * (NT / 32);                                         // 8 indices
      if (lane == 0) {
        wk[wig] = ((unsigned long long)mhi << 32) | mlo;
        wi[wig] = widx;
      }
      __syncthreads();
      if (tid == 0) {
        unsigned long long bk = wk[0];
        int bi = wi[0];
        for (int w = 1; w < NT / 32; ++w)
          if (wi[w] != 0x7fffffff && (bi == 0x7fffffff || wk[w] > bk || (wk[w] == bk && wi[w] < bi))) {
            bk = wk[w];
            bi = wi[w];
          }
        hdr[0] = bi;
        ipiv[gj] = gj + bi + 1;
      }
    }
    __syncthreads();
    const int jp = hdr[0];
    const T piv = colc[c + jp];
    const bool nonsingular = is_nonzero(piv);
    if (nonsingular && jp != 0)
      for (int t = c + tid; t < jb; t += NT) {
        T* col = P + t * RS;
        const T a = col[c];
        col[c] = col[c + jp];
        col[c + jp] = a;
      }
    __syncthreads();
    if (nonsingular) {
      const T rcp = T(1) / piv;
      for (int r = 1 + tid; r <= km; r += NT) colc[c + r] = rcp * colc[c + r];
    } else if (inf == 0) {
      inf = gj + 1;
    }
    __syncthreads();
    if (nonsingular) {  // rank-1 update of the panel's later columns: a thread per row
      for (int r = c + 1 + tid; r <= c + km; r += NT) {
        const T l = colc[r];
        for (int cc = c + 1; cc < jb; ++cc) {
          T* col = P + cc * RS;
          const T u = col[c];
          if (is_nonzero(u)) col[r] = fma(l, -u, col[r]);
        }
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < R * jb; e += NT) {
    const int c = e / R, r = e - c * R;
    const i64 g = sidx(r, c);
    if (g >= 0) ab[g] = P[c * RS + r];
  }
  if (tid == 0) *info = inf;
}

// One warp per column t = first + warp index: rows j0 .. j0+R-1 of the column replay
// the panel's steps.  smem: the panel's multipliers (R x jb, staged per CTA) and one
// R-row column buffer per warp.
template <typename T>
__global__ void __launch_bounds__(32 * kWideWarps) gbtrf_replay_kernel(i64 m, i64 n, int kl, int ku, i64 j0,
                                                                       i64 first, i64 last, T* ab, i64 ldab,
                                                                       const i64* ipiv) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int NB = kNB;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int kv = kl + ku, R = kl + NB, RS = R | 1;
  const i64 mn = min(m, n);
  const int jb = (int)min((i64)NB, mn - j0);
  T* L = reinterpret_cast<T*>(smem_raw);  // column k of the panel: L[k*RS + r], rows j0 + r
  T* colbuf = L + (i64)RS * NB + (i64)w * RS;
  __shared__ int st[kNB];
  for (int e = threadIdx.x; e < R * jb; e += blockDim.x) {
    const int k = e / R, r = e - k * R;
    const i64 i = j0 + r, col = j0 + k, d = i - col;
    L[k * RS + r] = (i < m && d >= -kv && d <= kl) ? ab[(kv + d) + col * ldab] : T(0);
  }
  if (threadIdx.x < jb) {  // -1: zero pivot (no interchange, no update)
    const i64 gj = j0 + threadIdx.x;
    st[threadIdx.x] = is_nonzero(ab[kv + gj * ldab]) ? (int)(ipiv[gj] - 1 - gj) : -1;
  }
  __syncthreads();
  for (i64 t = first + (i64)blockIdx.x * kWideWarps + w; t < last; t += (i64)gridDim.x * kWideWarps) {
    // the column's rows j0 .. j0+R-1 (zero outside the storage)
    for (int r = lane; r < R; r += 32) {
      const i64 i = j0 + r, d = i - t;
      colbuf[r] = (i < m && d >= -kv && d <= kl) ? ab[(kv + d) + t * ldab] : T(0);
    }
    __syncwarp();
    for (int k = 0; k < jb; ++k) {
      const int jp = st[k];
      if (jp < 0) continue;  // zero pivot: no interchange, no update
      T u = colbuf[k];
      if (jp != 0) {
        const T v = colbuf[k + jp];
        __syncwarp();
        if (lane == 0) {
          colbuf[k + jp] = u;
          colbuf[k] = v;
        }
        u = v;
      }
      __syncwarp();
      if (is_nonzero(u)) {
        const int km = (int)min((i64)kl, m - 1 - (j0 + k));
        const T nu = -u;
        const T* lk = L + k * RS;
        // rows k+1+lane, +32, ...: eight loads issued before their fmas
        int r = k + 1 + lane;
        for (; r + 7 * 32 <= k + km; r += 8 * 32) {
          T lv[8], av[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            lv[q] = lk[r + 32 * q];
            av[q] = colbuf[r + 32 * q];
          }
#pragma unroll
          for (int q = 0; q < 8; ++q) colbuf[r + 32 * q] = fma(lv[q], nu, av[q]);
        }
        for (; r <= k + km; r += 32) colbuf[r] = fma(lk[r], nu, colbuf[r]);
      }
      __syncwarp();
    }
    for (int r = lane; r < R; r += 32) {
      const i64 i = j0 + r, d = i - t;
      if (i < m && d >= -kv && d <= kl) ab[(kv + d) + t * ldab] = colbuf[r];
    }
    __syncwarp();
  }
}

template <typename T>
static int gbtrf_wide_impl(i64 m, i64 n, i64 kl, i64 ku, T* ab, i64 ldab, i64* ipiv, i64* info, cudaStream_t stream,
                           const char* name) {
  const int R = (int)kl + kNB, RS = R | 1;
  const i64 pbytes = (i64)RS * kNB * (i64)sizeof(T) + 256;  // panel + header (pivot, 8 warp keys/indices)
  const i64 rbytes = ((i64)RS * kNB + (i64)RS * kWideWarps) * (i64)sizeof(T);
  if (pbytes > 227 * 1024 || rbytes > 227 * 1024) {
    set_error("%s: band (kl=%lld) exceeds the panel limit", name, (long long)kl);
    return BM_ERR_UNSUPPORTED;
  }
  int r = cuda_status(ensure_smem((const void*)gbtrf_panel_kernel<T>, (int)pbytes), name);
  if (r) return r;
  r = cuda_status(ensure_smem((const void*)gbtrf_replay_kernel<T>, (int)rbytes), name);
  if (r) return r;
  r = cuda_status(cudaMemsetAsync(info, 0, sizeof(i64), stream), name);
  if (r) return r;
  if (kl > 0) {
    const i64 blocks = std::min<i64>(ceil_div(n * kl, 256), (i64)num_sms() * 16);
    zero_fill_kernel<T><<<(unsigned)blocks, 256, 0, stream>>>(n, (int)kl, ab, ldab);
    if ((r = launch_status(name))) return r;
  }
  const i64 mn = std::min(m, n);
  for (i64 j0 = 0; j0 < mn; j0 += kNB) {
    const i64 jb = std::min<i64>(kNB, mn - j0);
    gbtrf_panel_kernel<T><<<1, 256, (int)pbytes, stream>>>(m, n, (int)kl, (int)ku, j0, ab, ldab, ipiv, info);
    if ((r = launch_status(name))) return r;
    const i64 first = j0 + jb, last = std::min(n, j0 + jb + kl + ku);
    if (last > first) {
      const i64 blocks = std::min<i64>(ceil_div(last - first, kWideWarps), (i64)num_sms() * 2);
      gbtrf_replay_kernel<T><<<(unsigned)blocks, 32 * kWideWarps, (int)rbytes, stream>>>(
          m, n, (int)kl, (int)ku, j0, first, last, ab, ldab, ipiv);
      if ((r = launch_status(name))) return r;
    }
  }
  return BM_OK;
}

// Factor + solve of one system of a batch by a group of G warps.
template <typename T, int G>
__device__ __forceinline__ void gbsv_system(const bm_gb_desc& d, int s, T* AB, i64* ipiv, T* B, i64* info, T* smem) {
  T* ab = AB + d.ab_offset;
  i64* ip = ipiv + d.ipiv_offset;
  const int kl = (int)d.kl, ku = (int)d.ku, tid = Grp<G>::tid();
  // the register window where the band fits the group; its solve sweeps for Float32
  // (for Float64 the staged sweeps keep more of the FP64 pipe busy)
  const i64 r = reg_fits<T>(kl, ku, 32 * G)
                    ? gbtrf_reg_any<T, 32 * G>(d.n, d.n, kl, ku, ab, d.ldab, ip, smem, tid, 32 * G, G > 1)
                    : gbtrf_group<T, kP, G>(d.n, d.n, kl, ku, ab, d.ldab, ip, smem);
  if (tid == 0) info[s] = r;
  Grp<G>::sync();
  if (r == 0) {
    if (sizeof(T) == 4 && reg_solve_fits<T>(kl, ku)) {
      if ((tid >> 5) == 0)
        gbtrs_reg_any<T, kMaxRhs>(d.n, kl, ku, (int)d.nrhs, ab, d.ldab, ip, B + d.b_offset, d.ldb, smem, tid & 31);
    } else {
      gbtrs_all<T, G>(false, d.n, kl, ku, d.nrhs, ab, d.ldab, ip, B + d.b_offset, d.ldb, smem);
    }
  }
  Grp<G>::sync();
}

// Persistent batched factor + solve with a two-part schedule.  `order` lists the
// systems, wide ones first (most expensive first within each part).  Part 1: the
// CTA (W warps) takes the next wide system from the work queue (an atomic counter
// over `order`) and solves it as one group.  Part 2: once the queue reaches
// order[n_wide], each warp takes narrow systems on its own, in a shared-memory slice
// of narrow_elems elements.  Every system is factored in place and its right-hand
// sides solved; info[s] receives its gbtrf info.  A descriptor that is illegal, or
// whose band exceeds the bounds its part's shared memory was sized for (wkl/wku,
// nkl/nku), gets info[s] = -(field number) and is skipped; an order entry outside
// [0, count) is skipped.
template <typename T, int W>
__global__ void __launch_bounds__(32 * W) gbsv_batched_kernel(i64 count, const bm_gb_desc* __restrict__ descs,
                                                             const int32_t* __restrict__ order, i64 n_wide, T* AB,
                                                             i64* ipiv, T* B, i64* info, int32_t* counter,
                                                             i64 narrow_elems, i64 wkl, i64 wku, i64 nkl, i64 nku) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* base = reinterpret_cast<T*>(smem_raw);
  int idx;
  for (;;) {
    idx = next_item<W>(counter, reinterpret_cast<int*>(base));
    if (idx >= n_wide) break;
    const int s = order ? order[idx] : idx;
    if (s < 0 || s >= count) continue;
    const i64 bad = desc_check(descs[s], wkl, wku);
    if (bad) {
      if (threadIdx.x == 0) info[s] = bad;
      continue;
    }
    gbsv_system<T, W>(descs[s], s, AB, ipiv, B, info, base);
    __syncthreads();
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* ws = base + w * narrow_elems;
  int my = w == 0 ? idx : -1;  // the CTA's first narrow system goes to warp 0
  for (;;) {
    if (my < 0) {
      int v = 0;
      if (lane == 0) v = atomicAdd(counter, 1);
      my = __shfl_sync(0xffffffffu, v, 0);
    }
    if (my >= count) break;
    const int s = order ? order[my] : my;
    my = -1;
    if (s < 0 || s >= count) continue;
    const i64 bad = desc_check(descs[s], nkl, nku);
    if (bad) {
      if (lane == 0) info[s] = bad;
      continue;
    }
    gbsv_system<T, 1>(descs[s], s, AB, ipiv, B, info, ws);
  }
}

// One group of G warps per system pays off once the window holds a few hundred entries.
inline bool use_cta_group(i64 kl, i64 ku) { return (kl + 1) * (kl + ku + 1) >= 512; }

template <typename T>
static int gbtrf_impl(i64 m, i64 n, i64 kl, i64 ku, T* ab, i64 ldab, i64* ipiv, i64* info, cudaStream_t stream,
                      const char* name) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (kl < 0) return -3;
  if (ku < 0) return -4;
  if (ldab < 2 * kl + ku + 1) return -6;
  if (!info) return -8;
  if (m == 0 || n == 0) return cuda_status(cudaMemsetAsync(info, 0, sizeof(i64), stream), name);
  if (!ipiv) return -7;
  // bands whose window fits the register file: one lane per window column
  if (reg_class<T>(kl, ku)) return gbtrf_reg_run<T>(m, n, kl, ku, ab, ldab, ipiv, info, stream, name);
  const i64 bytes = gbtrf_smem_elems<kP>((int)kl, (int)ku) * (i64)sizeof(T);
  const i64 bbytes = gbtrf_blocked_smem_elems<T>((int)kl, (int)ku) * (i64)sizeof(T);
  // the one-column step where its window fits (measured faster); panels of kNB
  // columns where only the panel window fits
  if (bytes > 227 * 1024 && bbytes <= 227 * 1024) {
    if (kl + ku + 1 > 128) {
      int r = cuda_status(ensure_smem((const void*)gbtrf_blocked_one_kernel<T, 8>, (int)bbytes), name);
      if (r) return r;
      gbtrf_blocked_one_kernel<T, 8><<<1, 256, (int)bbytes, stream>>>(m, n, (int)kl, (int)ku, ab, ldab, ipiv, info);
    } else {
      int r = cuda_status(ensure_smem((const void*)gbtrf_blocked_one_kernel<T, 4>, (int)bbytes), name);
      if (r) return r;
      gbtrf_blocked_one_kernel<T, 4><<<1, 128, (int)bbytes, stream>>>(m, n, (int)kl, (int)ku, ab, ldab, ipiv, info);
    }
    return launch_status(name);
  }
  if (bytes > 227 * 1024) return gbtrf_wide_impl<T>(m, n, kl, ku, ab, ldab, ipiv, info, stream, name);
  if (use_cta_group(kl, ku) && kl + ku + 1 > 128) {  // one thread per window column
    int r = cuda_status(ensure_smem((const void*)gbtrf_one_kernel<T, 8>, (int)bytes), name);
    if (r) return r;
    gbtrf_one_kernel<T, 8><<<1, 256, (int)bytes, stream>>>(m, n, (int)kl, (int)ku, ab, ldab, ipiv, info);
  } else if (use_cta_group(kl, ku)) {
    int r = cuda_status(ensure_smem((const void*)gbtrf_one_kernel<T, 4>, (int)bytes), name);
    if (r) return r;
    gbtrf_one_kernel<T, 4><<<1, 128, (int)bytes, stream>>>(m, n, (int)kl, (int)ku, ab, ldab, ipiv, info);
  } else {
    int r = cuda_status(ensure_smem((const void*)gbtrf_one_kernel<T, 1>, (int)bytes), name);
    if (r) return r;
    gbtrf_one_kernel<T, 1><<<1, 32, (int)bytes, stream>>>(m, n, (int)kl, (int)ku, ab, ldab, ipiv, info);
  }
  return launch_status(name);
}

template <typename T>
static int gbtrs_impl(char trans, i64 n, i64 kl, i64 ku, i64 nrhs, const T* ab, i64 ldab, const i64* ipiv, T* B,
                      i64 ldb, cudaStream_t stream, const char* name) {
  const bool notr = (trans == 'N' || trans == 'n');
  if (!notr && !(trans == 'T' || trans == 't' || trans == 'C' || trans == 'c')) return -1;
  if (n < 0) return -2;
  if (kl < 0) return -3;
  if (ku < 0) return -4;
  if (nrhs < 0) return -5;
  if (ldab < 2 * kl + ku + 1) return -7;
  if (ldb < std::max<i64>(1, n)) return -10;
  if (n == 0 || nrhs == 0) return BM_OK;
  // the register-window sweeps (one warp per 32 right-hand sides) where the band fits
  if (notr && sizeof(T) == 4 && reg_solve_fits<T>(kl, ku))
    return gbtrs_reg_run<T>(n, kl, ku, nrhs, ab, ldab, ipiv, B, ldb, stream, name);
  const int ch = gbtrs_chunk_for<T>((int)kl, (int)ku, 227 * 1024);
  if (ch == 0) {
    set_error("%s: band too wide for the staged solve", name);
    return BM_ERR_UNSUPPORTED;
  }
  const i64 bytes = gbtrs_smem_elems((int)kl, (int)ku, ch) * (i64)sizeof(T);
  const i64 grid = std::min<i64>(ceil_div(nrhs, kMaxRhs), 65535);
  if (kl + ku >= 192) {  // wide: the CTA's 8 warps share the rows of few right-hand sides
    int r = cuda_status(ensure_smem((const void*)gbtrs_one_kernel<T, 8>, (int)bytes), name);
    if (r) return r;
    gbtrs_one_kernel<T, 8><<<(unsigned)grid, 256, (int)bytes, stream>>>(!notr, n, (int)kl, (int)ku, nrhs, ab, ldab,
                                                                         ipiv, B, ldb, ch);
  } else if ((kl + ku + 1) * std::min<i64>(nrhs, kMaxRhs) >= 256) {
    int r = cuda_status(ensure_smem((const void*)gbtrs_one_kernel<T, 4>, (int)bytes), name);
    if (r) return r;
    gbtrs_one_kernel<T, 4><<<(unsigned)grid, 128, (int)bytes, stream>>>(!notr, n, (int)kl, (int)ku, nrhs, ab, ldab,
                                                                         ipiv, B, ldb, ch);
  } else {
    int r = cuda_status(ensure_smem((const void*)gbtrs_one_kernel<T, 1>, (int)bytes), name);
    if (r) return r;
    gbtrs_one_kernel<T, 1><<<(unsigned)grid, 32, (int)bytes, stream>>>(!notr, n, (int)kl, (int)ku, nrhs, ab, ldab,
                                                                        ipiv, B, ldb, ch);
  }
  return launch_status(name);
}

// Shared memory of one group (NLMAX lanes) solving systems up to (kl, ku), 16-byte
// rounded, in T.
template <typename T, int NLMAX>
static i64 group_elems(i64 kl, i64 ku) {
  const i64 e = std::max(std::max(gbtrf_smem_elems<kP>((int)kl, (int)ku), gbtrs_smem_elems((int)kl, (int)ku)),
                         (i64)((reg_group_bytes<T, NLMAX, kMaxRhs>(kl, ku) + (long long)sizeof(T) - 1) / (long long)sizeof(T)));
  return ((e * (i64)sizeof(T) + 15) / 16) * 16 / (i64)sizeof(T);
}

template <typename T, int W>
static int gbsv_batched_launch(i64 count, const bm_gb_desc* descs, const int32_t* order, const bm_gb_schedule& sc,
                               T* AB, i64* ipiv, T* B, i64* info, int32_t* counter, cudaStream_t stream,
                               const char* name) {
  const i64 we = sc.n_wide > 0 ? group_elems<T, 32 * W>(sc.wide_kl, sc.wide_ku) : 0;
  const i64 ne = sc.n_wide < count ? group_elems<T, 32>(sc.narrow_kl, sc.narrow_ku) : 0;
  const i64 elems = std::max(std::max(we, W * ne), (i64)kHdr);
  const i64 bytes = elems * (i64)sizeof(T);
  if (bytes > 227 * 1024) {
    set_error("%s: the schedule's shared memory (%lld bytes) exceeds the per-CTA limit", name, (long long)bytes);
    return BM_ERR_UNSUPPORTED;
  }
  const void* kfn = (const void*)gbsv_batched_kernel<T, W>;
  int r = cuda_status(ensure_smem(kfn, (int)bytes), name);
  if (r) return r;
  int per_sm = 0;
  r = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gbsv_batched_kernel<T, W>, 32 * W, (int)bytes),
                  name);
  if (r) return r;
  per_sm = std::max(per_sm, 1);
  const i64 need = sc.n_wide + ceil_div(count - sc.n_wide, (i64)W);
  const i64 grid = std::min<i64>((i64)num_sms() * per_sm, std::max<i64>(need, 1));
  r = cuda_status(cudaMemsetAsync(counter, 0, sizeof(int32_t), stream), name);
  if (r) return r;
  gbsv_batched_kernel<T, W><<<(unsigned)grid, 32 * W, (int)bytes, stream>>>(
      count, descs, order, sc.n_wide, AB, ipiv, B, info, counter, ne, sc.wide_kl, sc.wide_ku, sc.narrow_kl,
      sc.narrow_ku);
  return launch_status(name);
}

template <typename T>
static int gbsv_batched_sched_impl(i64 count, const bm_gb_desc* descs, const int32_t* order, const bm_gb_schedule* sc,
                                   T* AB, i64* ipiv, T* B, i64* info, int32_t* counter, cudaStream_t stream,
                                   const char* name) {
  if (count < 0) return -1;
  if (!descs && count) return -2;
  if (!sc) return -4;
  if (sc->n_wide < 0 || sc->n_wide > count || (sc->warps != 4 && sc->warps != 8) || sc->wide_kl < 0 ||
      sc->wide_ku < 0 || sc->narrow_kl < 0 || sc->narrow_ku < 0)
    return -4;
  if (!info && count) return -8;
  if (!counter) return -9;
  if (count == 0) return BM_OK;
  if (sc->warps == 8) return gbsv_batched_launch<T, 8>(count, descs, order, *sc, AB, ipiv, B, info, counter, stream, name);
  return gbsv_batched_launch<T, 4>(count, descs, order, *sc, AB, ipiv, B, info, counter, stream, name);
}

// The schedule of the single-part entry points: every system wide (one CTA of 4 warps
// each) when the widest window holds 512 entries or more, else every system narrow.
inline bm_gb_schedule default_schedule(i64 count, i64 max_kl, i64 max_ku) {
  bm_gb_schedule sc;
  sc.n_wide = use_cta_group(max_kl, max_ku) ? count : 0;
  sc.warps = 4;
  sc.wide_kl = sc.narrow_kl = max_kl;
  sc.wide_ku = sc.narrow_ku = max_ku;
  return sc;
}

template <typename T>
static int gbsv_batched_impl(i64 count, const bm_gb_desc* descs, const int32_t* order, T* AB, i64* ipiv, T* B,
                             i64* info, int32_t* counter, i64 max_kl, i64 max_ku, cudaStream_t stream,
                             const char* name) {
  // arguments in order (count 1, descs 2, order 3, AB 4, ipiv 5, B 6, info 7, counter 8,
  // max_kl 9, max_ku 10); the schedule built from them is then always valid
  if (count < 0) return -1;
  if (!descs && count) return -2;
  if (!info && count) return -7;
  if (!counter) return -8;
  if (max_kl < 0) return -9;
  if (max_ku < 0) return -10;
  const bm_gb_schedule sc = default_schedule(count, max_kl, max_ku);
  return gbsv_batched_sched_impl<T>(count, descs, order, &sc, AB, ipiv, B, info, counter, stream, name);
}

// ---------------------------------------------------------------------------
// Allocation-free batched solve.  Some callers of this library cannot call
// cudaMalloc at solve time: real-time loops that must not block on the allocator,
// and hosts whose device memory is owned by another runtime's pool (Julia's CUDA.jl,
// PyTorch) and that cannot hand the library a workspace.  For them, the scratch of the batched
// solve -- the work-queue counter and the longest-first processing order -- lives
// in this file-scope device array instead of caller-provided memory.  Every GPU that
// loads the library keeps these 256 KiB (plus 256 bytes) until the process exits.
constexpr int kNoAllocMaxSystems = 65536;
constexpr int kNoAllocHeader = 64;  // int32 slots before the order list; slot 0 = work counter
static __device__ __align__(256) int32_t g_noalloc_scratch[kNoAllocHeader + kNoAllocMaxSystems];

// Longest-first order of the systems, written to `order`: systems are binned by
// floor(log2(cost)) (cost as in lpt_order on the host) and emitted from the most
// expensive bin down.  Within a bin the order is arbitrary; each system's result does
// not depend on it.  One CTA; count <= kNoAllocMaxSystems.
__global__ void __launch_bounds__(1024) lpt_order_kernel(i64 count, const bm_gb_desc* __restrict__ descs,
                                                         int32_t* __restrict__ order) {
  __shared__ int hist[64];
  __shared__ int start[64];
  if (threadIdx.x < 64) hist[threadIdx.x] = 0;
  __syncthreads();
  auto bin_of = [&](i64 s) {
    const bm_gb_desc d = descs[s];
    const double cost = (double)d.n * (2.0 * d.kl * (d.kl + d.ku) + d.kl) +
                        2.0 * d.nrhs * d.n * (2.0 * d.kl + d.ku + 1) + 1.0;
    const int e = ilogb(cost);               // 0 .. 62
    return 63 - min(max(e, 0), 63);          // most expensive -> bin 0
  };
  for (i64 s = threadIdx.x; s < count; s += blockDim.x) atomicAdd(&hist[bin_of(s)], 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int b = 0; b < 64; ++b) {
      start[b] = acc;
      acc += hist[b];
    }
  }
  __syncthreads();
  for (i64 s = threadIdx.x; s < count; s += blockDim.x) order[atomicAdd(&start[bin_of(s)], 1)] = (int32_t)s;
}

// Device address of g_noalloc_scratch on the current device, looked up once per device
// and cached for the life of the process (a cudaDeviceReset invalidates it: the
// library must then be reloaded).
static int noalloc_scratch(int32_t** out, const char* name) {
  static std::mutex mu;
  static int32_t* cache[64] = {nullptr};
  int dev = 0;
  int r = cuda_status(cudaGetDevice(&dev), name);
  if (r) return r;
  if (dev < 0 || dev >= 64) {
    set_error("%s: device ordinal %d out of range", name, dev);
    return BM_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(mu);
  if (!cache[dev]) {
    int32_t* ptr = nullptr;
    r = cuda_status(cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch), name);
    if (r) return r;
    cache[dev] = ptr;
  }
  *out = cache[dev];
  return BM_OK;
}

static int gbsv_batched_noalloc_impl(i64 count, const bm_gb_desc* descs, double* AB, i64* ipiv, double* B, i64* info,
                                     i64 max_kl, i64 max_ku, cudaStream_t stream, const char* name) {
  if (count < 0) return -1;
  if (!descs && count) return -2;
  if (!info && count) return -6;
  if (max_kl < 0) return -7;
  if (max_ku < 0) return -8;
  if (count > kNoAllocMaxSystems) {
    set_error("%s: %lld systems exceed the allocation-free limit of %d; use bm_dgbsv_batched", name,
              (long long)count, kNoAllocMaxSystems);
    return BM_ERR_UNSUPPORTED;
  }
  if (count == 0) return BM_OK;
  int32_t* scratch = nullptr;
  int r = noalloc_scratch(&scratch, name);
  if (r) return r;
  lpt_order_kernel<<<1, 1024, 0, stream>>>(count, descs, scratch + kNoAllocHeader);
  r = launch_status(name);
  if (r) return r;
  // the batched launch below resets the work counter (scratch[0]) before it starts
  return gbsv_batched_impl<double>(count, descs, scratch + kNoAllocHeader, AB, ipiv, B, info, scratch, max_kl, max_ku,
                                   stream, name);
}

}  // namespace bm

extern "C" int bm_dgbsv_batched_noalloc(int64_t count, const bm_gb_desc* descs, double* AB, int64_t* ipiv, double* B,
                                        int64_t* info, int64_t max_kl, int64_t max_ku, bm_stream_t stream) {
  return bm::gbsv_batched_noalloc_impl(count, descs, AB, ipiv, B, info, max_kl, max_ku,
                                       reinterpret_cast<cudaStream_t>(stream), "bm_dgbsv_batched_noalloc");
}

extern "C" int bm_dgbtrf(int64_t m, int64_t n, int64_t kl, int64_t ku, double* AB, int64_t ldab, int64_t* ipiv,
                         int64_t* info, bm_stream_t stream) {
  return bm::gbtrf_impl<double>(m, n, kl, ku, AB, ldab, ipiv, info, reinterpret_cast<cudaStream_t>(stream),
                                "bm_dgbtrf");
}
extern "C" int bm_sgbtrf(int64_t m, int64_t n, int64_t kl, int64_t ku, float* AB, int64_t ldab, int64_t* ipiv,
                         int64_t* info, bm_stream_t stream) {
  return bm::gbtrf_impl<float>(m, n, kl, ku, AB, ldab, ipiv, info, reinterpret_cast<cudaStream_t>(stream),
                               "bm_sgbtrf");
}
extern "C" int bm_dgbtrs(char trans, int64_t n, int64_t kl, int64_t ku, int64_t nrhs, const double* AB, int64_t ldab,
                         const int64_t* ipiv, double* B, int64_t ldb, bm_stream_t stream) {
  return bm::gbtrs_impl<double>(trans, n, kl, ku, nrhs, AB, ldab, ipiv, B, ldb,
                                reinterpret_cast<cudaStream_t>(stream), "bm_dgbtrs");
}
extern "C" int bm_sgbtrs(char trans, int64_t n, int64_t kl, int64_t ku, int64_t nrhs, const float* AB, int64_t ldab,
                         const int64_t* ipiv, float* B, int64_t ldb, bm_stream_t stream) {
  return bm::gbtrs_impl<float>(trans, n, kl, ku, nrhs, AB, ldab, ipiv, B, ldb,
                               reinterpret_cast<cudaStream_t>(stream), "bm_sgbtrs");
}
extern "C" int bm_dgbsv_batched_sched(int64_t count, const bm_gb_desc* descs, const int32_t* order,
                                      const bm_gb_schedule* sched, double* AB, int64_t* ipiv, double* B, int64_t* info,
                                      int32_t* counter, bm_stream_t stream) {
  return bm::gbsv_batched_sched_impl<double>(count, descs, order, sched, AB, ipiv, B, info, counter,
                                             reinterpret_cast<cudaStream_t>(stream), "bm_dgbsv_batched_sched");
}
extern "C" int bm_sgbsv_batched_sched(int64_t count, const bm_gb_desc* descs, const int32_t* order,
                                      const bm_gb_schedule* sched, float* AB, int64_t* ipiv, float* B, int64_t* info,
                                      int32_t* counter, bm_stream_t stream) {
  return bm::gbsv_batched_sched_impl<float>(count, descs, order, sched, AB, ipiv, B, info, counter,
                                            reinterpret_cast<cudaStream_t>(stream), "bm_sgbsv_batched_sched");
}
extern "C" int bm_dgbsv_batched(int64_t count, const bm_gb_desc* descs, const int32_t* order, double* AB,
                                int64_t* ipiv, double* B, int64_t* info, int32_t* counter, int64_t max_kl,
                                int64_t max_ku, bm_stream_t stream) {
  return bm::gbsv_batched_impl<double>(count, descs, order, AB, ipiv, B, info, counter, max_kl, max_ku,
                                       reinterpret_cast<cudaStream_t>(stream), "bm_dgbsv_batched");
}
extern "C" int bm_sgbsv_batched(int64_t count, const bm_gb_desc* descs, const int32_t* order, float* AB,
                                int64_t* ipiv, float* B, int64_t* info, int32_t* counter, int64_t max_kl,
                                int64_t max_ku, bm_stream_t stream) {
  return bm::gbsv_batched_impl<float>(count, descs, order, AB, ipiv, B, info, counter, max_kl, max_ku,
                                      reinterpret_cast<cudaStream_t>(stream), "bm_sgbsv_batched");
}
