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
// 128 or 512 in Float64): the factorization runs panel by panel over the gbtrf storage
// in global memory, as two launches per panel of NB columns (NB = 8 or 4, chosen by kl;
// 16 for the shared-memory panel).
//   * gbtrf_panel_reg_kernel (one CTA of 256 threads) holds the panel -- rows j0 ..
//     j0+kl+NB-1 of its NB columns -- in registers and takes dgbtf2's steps on it (see
//     below); gbtrf_panel_kernel does the same in shared memory for the widest bands.
//     Either stores the panel back (L in dgbtf2's format) with the pivots.
//   * gbtrf_replay_kernel (one CTA of kReplayNT threads per column, one warp per
//     sub-partition): every column the panel's steps can reach (up to kl+ku to its
//     right) replays the steps in order on its rows j0 .. j0+kl+NB-1, held in
//     registers (row r by thread r mod kReplayNT).  At each step the threads holding the
//     pivot row and row k publish both values through shared memory, one barrier, and
//     every thread applies the interchange and its rows' fmas; the multipliers are
//     staged once per CTA, and a step's interchange and zero-pivot flag come from ipiv
//     and the stored U(j,j).
// Each element therefore receives dgbtf2's sequence of operations: factors and pivots
// equal the unblocked result bit for bit.
constexpr int kPanelNT = 256;
constexpr int kReplayNT = 128;

// the top kl rows of gbtrf storage (fill-in) start at zero, as dgbtrf sets them
template <typename T>
__global__ void zero_fill_kernel(i64 n, int kl, T* ab, i64 ldab) {
  const i64 total = n * (i64)kl;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
    const i64 c = e / kl;
    ab[(e - c * kl) + c * ldab] = T(0);
  }
}

// Shared memory of the panel kernel: the panel (kNB columns of RS = (kl+kNB)|1
// elements) and a header (per-warp keys and indices, the reciprocal of the pivot).
template <typename T>
__host__ __device__ constexpr i64 panel_smem_bytes(int kl) {
  return (i64)((kl + kNB) | 1) * kNB * (i64)sizeof(T) + 256;
}

// Shared-memory panel, for bands whose panel rows exceed the register panels: the
// panel in shared memory, one thread per row for the scaling and the update.
template <typename T>
__global__ void __launch_bounds__(kPanelNT) gbtrf_panel_kernel(i64 m, i64 n, int kl, int ku, i64 j0, T* ab,
                                                                i64 ldab, i64* ipiv, i64* info) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int NT = kPanelNT, NB = kNB, NW = NT / 32;
  const int tid = threadIdx.x, lane = tid & 31, wig = tid >> 5;
  const int kv = kl + ku, R = kl + NB, RS = R | 1;
  const i64 mn = min(m, n);
  const int jb = (int)min((i64)NB, mn - j0);
  grid_dep_wait();  // the previous replay's columns
  grid_dep_launch();
  T* P = reinterpret_cast<T*>(smem_raw);  // panel: column c (0..jb-1) x row r (matrix row j0 + r)
  unsigned long long* wk = reinterpret_cast<unsigned long long*>(P + (i64)RS * NB);  // NW warp keys
  int* wi = reinterpret_cast<int*>(wk + NW);                                          // NW warp indices
  T* srcp = reinterpret_cast<T*>(wk + NW + NW / 2);                                   // 1 / pivot
  // entry (row j0+r, column j0+c) of the storage when it lies in it
  auto sidx = [&](int r, int c) -> i64 {
    const i64 i = j0 + r, col = j0 + c;
    const i64 d = i - col;
    return (i < m && d >= -kv && d <= kl) ? (kv + d) + col * ldab : (i64)-1;
  };
  for (int c = 0; c < jb; ++c)  // asynchronous element copies (zero outside the storage), one wait
    for (int r = tid; r < R; r += NT) {
      const i64 g = sidx(r, c);
      cp_async_elem(P + c * RS + r, g >= 0 ? ab + g : ab, g >= 0);
    }
  cp_async_commit();
  i64 inf = *info;
  cp_async_wait<0>();
  __syncthreads();
  for (int c = 0; c < jb; ++c) {
    const i64 gj = j0 + c;
    const int km = (int)min((i64)kl, m - 1 - gj);
    T* colc = P + c * RS;
    // idamax over rows c..c+km: a warp argmax (first index on ties), then the warps'
    // (key, index) pairs, combined the same way by every warp
    {
      unsigned long long key = 0ull;
      int idx = 0x7fffffff;
      for (int r = tid; r <= km; r += NT) {
        const unsigned long long k = pivot_key(colc[c + r], r == 0);
        if (idx == 0x7fffffff || k > key) {
          key = k;
          idx = r;
        }
      }
      const int widx = warp_argmax_first(key, idx);
      if (lane == 0) {
        wk[wig] = widx == 0x7fffffff ? 0ull : pivot_key(colc[c + widx], widx == 0);
        wi[wig] = widx;
      }
    }
    __syncthreads();
    const int jp = warp_argmax_first(lane < NW ? wk[lane] : 0ull, lane < NW ? wi[lane] : 0x7fffffff);
    const T piv = colc[c + jp];
    const bool ns = is_nonzero(piv);
    if (tid == 0) {
      ipiv[gj] = gj + jp + 1;
      if (ns) *srcp = T(1) / piv;
    }
    if (!ns && inf == 0) inf = gj + 1;
    // interchange of rows c and c+jp in the panel's later columns (warp 1); column c's
    // own interchange is folded into the scaling below
    if (ns && jp != 0 && tid >= 32 && tid - 32 < jb - 1 - c) {
      T* col = P + (c + 1 + tid - 32) * RS;
      const T a = col[c];
      col[c] = col[c + jp];
      col[c + jp] = a;
    }
    __syncthreads();
    if (ns) {  // multipliers and the rank-1 update of the panel's later columns, by row
      const T rcp = *srcp;
      const T d0 = colc[c];  // row c's value before the interchange: it moves to row c+jp
      for (int r = 1 + tid; r <= km; r += NT) {
        const T l = rcp * (r == jp ? d0 : colc[c + r]);
        colc[c + r] = l;
        for (int cc = c + 1; cc < jb; ++cc) {
          T* col = P + cc * RS;
          const T u = col[c];
          if (is_nonzero(u)) col[c + r] = fma(l, -u, col[c + r]);
        }
      }
    }
    __syncthreads();
    // U(j, j): written after the barrier, as the scaling above still reads row c's
    // old value; no thread reads column c again
    if (tid == 0 && ns) colc[c] = piv;
  }
  __syncthreads();
  for (int e = tid; e < R * jb; e += NT) {
    const int c = e / R, r = e - c * R;
    const i64 g = sidx(r, c);
    if (g >= 0) ab[g] = P[c * RS + r];
  }
  if (tid == 0) *info = inf;
}

// Register panel of NB columns (R = kl + NB <= RPT * kPanelNT rows): thread t holds rows
// t + kPanelNT*i of the panel's columns in registers, the column of the current step at index 0 (the
// window rotates by one column per step, and the finished column is stored).  A step:
// the key of each row, a warp argmax, the warps' results through shared memory (one
// barrier); the threads holding the pivot row and row c publish both rows and the
// reciprocal of the pivot (a second barrier); then every thread scales and updates its
// own rows.  One CTA, so the panel's steps cost two barriers each and no shared-memory
// traffic for the elements themselves.  (Measured against two alternatives at
// kl = 128: four warps with two rows per thread, 41 us per panel, and rows rotating
// out of the active slots with a uniform zero mask, 45 us, against 33 us for this one.)
template <typename T, int RPT, int NB>
__global__ void __launch_bounds__(kPanelNT) gbtrf_panel_reg_kernel(i64 m, i64 n, int kl, int ku, i64 j0, T* ab,
                                                                    i64 ldab, i64* ipiv, i64* info) {
  constexpr int NT = kPanelNT, NW = NT / 32;
  __shared__ unsigned long long wk[2][NW];
  __shared__ int wi[2][NW];
  __shared__ T prow[2][NB], crow[2][NB], srcp[2];
  const int tid = threadIdx.x, lane = tid & 31, wig = tid >> 5;
  const int kv = kl + ku, R = kl + NB;
  const i64 mn = min(m, n);
  const int jb = (int)min((i64)NB, mn - j0);
  grid_dep_wait();  // the previous replay's columns
  grid_dep_launch();
  T v[RPT][NB];  // v[i][q]: row tid + NT*i of column c + q at step c
#pragma unroll
  for (int i = 0; i < RPT; ++i)
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      const int r = tid + NT * i, d = r - q;
      const bool ok = q < jb && r < R && j0 + r < m && d >= -kv && d <= kl;
      v[i][q] = ok ? ab[(kv + d) + (j0 + q) * ldab] : T(0);
    }
  i64 inf = *info;
  for (int c = 0; c < jb; ++c) {
    const i64 gj = j0 + c;
    const int km = (int)min((i64)kl, m - 1 - gj);
    const int par = c & 1;
    // idamax over rows c..c+km (first index on ties)
    unsigned long long key = 0ull;
    int idx = 0x7fffffff;
#pragma unroll
    for (int i = 0; i < RPT; ++i) {
      const int r = tid + NT * i;
      if (r >= c && r <= c + km) {
        const unsigned long long k = pivot_key(v[i][0], r == c);
        if (idx == 0x7fffffff || k > key) {
          key = k;
          idx = r - c;
        }
      }
    }
    const int widx = warp_argmax_first(key, idx);
    const int src = widx == 0x7fffffff ? 0 : (c + widx) & 31;  // the lane holding the winner
    const unsigned long long wkey = __shfl_sync(0xffffffffu, key, src);
    if (lane == 0) {
      wk[par][wig] = widx == 0x7fffffff ? 0ull : wkey;
      wi[par][wig] = widx;
    }
    __syncthreads();
    const int jp = warp_argmax_first(lane < NW ? wk[par][lane] : 0ull, lane < NW ? wi[par][lane] : 0x7fffffff);
    const int rp = c + jp;
    // the pivot row and row c (columns c .. c+NB-1 of the window), and 1/pivot
#pragma unroll
    for (int i = 0; i < RPT; ++i) {
      const int r = tid + NT * i;
      if (r == rp) {
#pragma unroll
        for (int q = 0; q < NB; ++q) prow[par][q] = v[i][q];
        if (is_nonzero(v[i][0])) srcp[par] = T(1) / v[i][0];
      }
      if (r == c && jp != 0) {
#pragma unroll
        for (int q = 0; q < NB; ++q) crow[par][q] = v[i][q];
      }
    }
    if (tid == 0) ipiv[gj] = gj + jp + 1;
    __syncthreads();
    const bool ns = is_nonzero(prow[par][0]);
    if (!ns && inf == 0) inf = gj + 1;
    if (ns) {
      const T rcp = srcp[par];
      const int nq = jb - c;  // columns of the panel from c on
      T u[NB];
#pragma unroll
      for (int q = 1; q < NB; ++q) u[q] = prow[par][q];
#pragma unroll
      for (int i = 0; i < RPT; ++i) {
        const int r = tid + NT * i;
        if (r == c) {  // row c takes the pivot row
#pragma unroll
          for (int q = 0; q < NB; ++q) v[i][q] = prow[par][q];
        } else if (r > c && r <= c + km) {
          const bool sw = r == rp;  // this row takes row c's values
          const T l = rcp * (sw ? crow[par][0] : v[i][0]);
          v[i][0] = l;
#pragma unroll
          for (int q = 1; q < NB; ++q)
            if (q < nq) {
              const T a = sw ? crow[par][q] : v[i][q];
              v[i][q] = is_nonzero(u[q]) ? fma(l, -u[q], a) : a;
            }
        }
      }
    }
    // column c is final: store it and rotate the window
#pragma unroll
    for (int i = 0; i < RPT; ++i) {
      const int r = tid + NT * i, d = r - c;
      if (r < R && j0 + r < m && d >= -kv && d <= kl) ab[(kv + d) + gj * ldab] = v[i][0];
#pragma unroll
      for (int q = 0; q < NB - 1; ++q) v[i][q] = v[i][q + 1];
      v[i][NB - 1] = T(0);
    }
  }
  if (tid == 0) *info = inf;
}

// One CTA per column t = first + blockIdx.x; thread r mod kReplayNT holds rows j0 + r
// (RPT of them) in registers.  smem: the panel's multipliers, L[k*RS + r] for the row
// j0 + r at step k.
template <typename T>
__host__ __device__ constexpr i64 replay_smem_bytes(int kl, int nb) {
  return (i64)((kl + nb) | 1) * nb * (i64)sizeof(T);
}

template <typename T, int RPT, int NB>
__global__ void __launch_bounds__(kReplayNT) gbtrf_replay_kernel(i64 m, i64 n, int kl, int ku, i64 j0, i64 first,
                                                                  T* ab, i64 ldab, const i64* ipiv) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int NT = kReplayNT;
  __shared__ int st[NB];
  __shared__ T xch[2][2];  // [step parity][0: the pivot row's value, 1: row k's value]
  const int tid = threadIdx.x;
  const int kv = kl + ku, R = kl + NB, RS = R | 1;
  const i64 mn = min(m, n);
  const int jb = (int)min((i64)NB, mn - j0);
  const i64 t = first + blockIdx.x;
  T* L = reinterpret_cast<T*>(smem_raw);
  T v[RPT];
#pragma unroll
  for (int i = 0; i < RPT; ++i) {
    const int r = tid + NT * i;
    const i64 row = j0 + r, d = row - t;
    v[i] = (r < R && row < m && d >= -kv && d <= kl) ? ab[(kv + d) + t * ldab] : T(0);
  }
  // the column is complete (the previous replay ended before the panel began); the
  // panel's multipliers and pivots are waited for
  grid_dep_launch();
  grid_dep_wait();
  for (int k = 0; k < jb; ++k) {  // asynchronous element copies, one wait
    const i64 gk = j0 + k;
    const int km = (int)min((i64)kl, m - 1 - gk);
    for (int i = tid; i < km; i += NT) cp_async_elem(L + k * RS + k + 1 + i, ab + (kv + 1 + i) + gk * ldab, true);
  }
  cp_async_commit();
  if (tid < jb) {  // -1: zero pivot (no interchange, no update)
    const i64 gj = j0 + tid;
    st[tid] = is_nonzero(ab[kv + gj * ldab]) ? (int)(ipiv[gj] - 1 - gj) : -1;
  }
  cp_async_wait<0>();
  __syncthreads();
  for (int k = 0; k < jb; ++k) {
    const int jp = st[k];
    if (jp < 0) continue;  // the same for every thread
    const int par = k & 1;
#pragma unroll
    for (int i = 0; i < RPT; ++i) {
      const int r = tid + NT * i;
      if (r == k + jp) xch[par][0] = v[i];
      if (r == k) xch[par][1] = v[i];
    }
    __syncthreads();
    const T u = xch[par][0], a0 = xch[par][1];
    const bool doit = is_nonzero(u);
    const int km = (int)min((i64)kl, m - 1 - (j0 + k));
    const T* lk = L + k * RS;
#pragma unroll
    for (int i = 0; i < RPT; ++i) {
      const int r = tid + NT * i;
      if (r == k) {
        v[i] = u;
      } else if (r > k && r <= k + km) {
        T a = r == k + jp ? a0 : v[i];
        if (doit) a = fma(lk[r], -u, a);
        v[i] = a;
      }
    }
  }
#pragma unroll
  for (int i = 0; i < RPT; ++i) {
    const int r = tid + NT * i;
    const i64 row = j0 + r, d = row - t;
    if (r < R && row < m && d >= -kv && d <= kl) ab[(kv + d) + t * ldab] = v[i];
  }
}

// rows held per replay thread: a class >= ceil((kl + nb) / kReplayNT)
inline int replay_rpt(i64 kl, int nb) {
  const i64 r = ceil_div(kl + nb, (i64)kReplayNT);
  return r <= 1 ? 1 : r <= 2 ? 2 : r <= 3 ? 3 : r <= 4 ? 4 : r <= 5 ? 5 : r <= 6 ? 6 : r <= 8 ? 8 : r <= 12 ? 12 : 16;
}

// Launch with programmatic stream serialization: the kernel may begin while the previous
// one in the stream finishes, and waits for it with grid_dep_wait() before reading its
// results.
template <typename... KArgs, typename... Args>
static cudaError_t launch_dependent(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem,
                                    cudaStream_t stream, Args... args) {
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

template <typename T, int NB>
static int gbtrf_wide_run(i64 m, i64 n, i64 kl, i64 ku, T* ab, i64 ldab, i64* ipiv, i64* info, cudaStream_t stream,
                          const char* name) {
  const i64 pbytes = panel_smem_bytes<T>((int)kl), rbytes = replay_smem_bytes<T>((int)kl, NB);
  if (pbytes > 227 * 1024 || kl + NB > 16 * kReplayNT) {
    set_error("%s: band (kl=%lld) exceeds the panel limit", name, (long long)kl);
    return BM_ERR_UNSUPPORTED;
  }
  const int rpt = replay_rpt(kl, NB);
  // f(kernel) for the replay kernel of this band's row class
  auto with_replay = [&](auto&& f) {
    switch (rpt) {
#define BM_RPT(v) \
  case v:         \
    return f(gbtrf_replay_kernel<T, v, NB>);
      BM_RPT(1) BM_RPT(2) BM_RPT(3) BM_RPT(4) BM_RPT(5) BM_RPT(6) BM_RPT(8) BM_RPT(12)
#undef BM_RPT
      default:
        return f(gbtrf_replay_kernel<T, 16, NB>);
    }
  };
  // the register panel where the panel's rows fit RPT rows per thread (at most 3 in
  // Float64, 4 in Float32, within the register file); else the shared-memory panel
  const int prpt_need = (int)ceil_div(kl + NB, (i64)kPanelNT);
  const int prpt = prpt_need <= (sizeof(T) == 8 ? 3 : 4) ? prpt_need : 0;
  if (!prpt && NB != kNB) {  // the shared-memory panel is kNB columns wide
    set_error("%s: internal panel width %d without a register panel", name, NB);
    return BM_ERR_UNSUPPORTED;
  }
  int r = cuda_status(ensure_smem((const void*)gbtrf_panel_kernel<T>, (int)pbytes), name);
  if (r) return r;
  r = cuda_status(with_replay([&](auto kern) { return ensure_smem((const void*)kern, (int)rbytes); }), name);
  if (r) return r;
  r = cuda_status(cudaMemsetAsync(info, 0, sizeof(i64), stream), name);
  if (r) return r;
  if (kl > 0) {
    const i64 blocks = std::min<i64>(ceil_div(n * kl, 256), (i64)num_sms() * 16);
    zero_fill_kernel<T><<<(unsigned)blocks, 256, 0, stream>>>(n, (int)kl, ab, ldab);
    if ((r = launch_status(name))) return r;
  }
  const i64 mn = std::min(m, n);
  for (i64 j0 = 0; j0 < mn; j0 += NB) {
    const i64 jb = std::min<i64>(NB, mn - j0);
    cudaError_t le;
    switch (prpt) {
      case 1:
        le = launch_dependent(gbtrf_panel_reg_kernel<T, 1, NB>, 1, kPanelNT, 0, stream, m, n, (int)kl, (int)ku, j0, ab,
                              ldab, ipiv, info);
        break;
      case 2:
        le = launch_dependent(gbtrf_panel_reg_kernel<T, 2, NB>, 1, kPanelNT, 0, stream, m, n, (int)kl, (int)ku, j0, ab,
                              ldab, ipiv, info);
        break;
      case 3:
        le = launch_dependent(gbtrf_panel_reg_kernel<T, 3, NB>, 1, kPanelNT, 0, stream, m, n, (int)kl, (int)ku, j0, ab,
                              ldab, ipiv, info);
        break;
      case 4:
        if constexpr (sizeof(T) == 4) {
          le = launch_dependent(gbtrf_panel_reg_kernel<T, 4, NB>, 1, kPanelNT, 0, stream, m, n, (int)kl, (int)ku, j0,
                                ab, ldab, ipiv, info);
          break;
        }
        [[fallthrough]];
      default:
        le = launch_dependent(gbtrf_panel_kernel<T>, 1, kPanelNT, (size_t)pbytes, stream, m, n, (int)kl, (int)ku, j0,
                              ab, ldab, ipiv, info);
    }
    if ((r = cuda_status(le, name))) return r;
    if ((r = launch_status(name))) return r;
    const i64 first = j0 + jb, last = std::min(n, j0 + jb + kl + ku);
    if (last > first) {
      r = cuda_status(with_replay([&](auto kern) {
                        return launch_dependent(kern, (unsigned)(last - first), kReplayNT, (size_t)rbytes, stream, m, n,
                                                (int)kl, (int)ku, j0, first, ab, ldab, ipiv);
                      }),
                      name);
      if (r) return r;
      if ((r = launch_status(name))) return r;
    }
  }
  return BM_OK;
}

// Panel width of the wide-band factorization: the panel's bulk update grows with the
// width (about (NB-1)/2 columns x kl rows per step, on one SM), the launches per column
// shrink with it.  Measured (Float64, GB300): kl = 128 -> 2.46 / 1.97 / 2.08 us per column
// for NB = 16 / 8 / 4; kl = 512 -> 7.31 / 5.10 / 4.48.  Bands too wide for the register
// panel take the 16-column shared-memory panel.
template <typename T>
static int gbtrf_wide_impl(i64 m, i64 n, i64 kl, i64 ku, T* ab, i64 ldab, i64* ipiv, i64* info, cudaStream_t stream,
                           const char* name) {
  const int maxr = sizeof(T) == 8 ? 3 : 4;
  if (kl > 256 && ceil_div(kl + 4, (i64)kPanelNT) <= maxr)
    return gbtrf_wide_run<T, 4>(m, n, kl, ku, ab, ldab, ipiv, info, stream, name);
  if (ceil_div(kl + 8, (i64)kPanelNT) <= maxr)
    return gbtrf_wide_run<T, 8>(m, n, kl, ku, ab, ldab, ipiv, info, stream, name);
  return gbtrf_wide_run<T, kNB>(m, n, kl, ku, ab, ldab, ipiv, info, stream, name);
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
// The Float64 4-warp variant is held to three CTAs per SM (at most 170 registers a
// thread): with more registers the CTAs per SM drop to two, which costs a quarter of the
// batch's throughput.  (Float32 would spill at that bound.)
template <typename T, int W>
__global__ void __launch_bounds__(32 * W, (W == 4 && sizeof(T) == 8) ? 3 : 1)
    gbsv_batched_kernel(i64 count, const bm_gb_desc* __restrict__ descs, const int32_t* __restrict__ order,
                        i64 n_wide, T* AB, i64* ipiv, T* B, i64* info, int32_t* counter, i64 narrow_elems, i64 wkl,
                        i64 wku, i64 nkl, i64 nku) {
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
  // tiny bands: one warp, a lane per window element
  if (tiny_fits(kl, ku)) return gbtrf_tiny_run<T>(m, n, kl, ku, ab, ldab, ipiv, info, stream, name);
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
  // tiny bands: a warp per right-hand side, a lane per window row
  if (notr && tiny_solve_fits(kl, ku)) return gbtrs_tiny_run<T>(n, kl, ku, nrhs, ab, ldab, ipiv, B, ldb, stream, name);
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
