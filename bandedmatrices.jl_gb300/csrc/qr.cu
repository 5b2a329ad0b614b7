// Banded Householder QR and its Q / Q' application (replaces _banded_qr! and
// banded_qr_lmul!, src/banded/bandedqr.jl:13-28 and :38-94), plus the upper
// triangular band solve that finishes qr(A) \ b (tbsv!, src/blas.jl:112-147, reached
// through src/tribanded.jl:75-83).
//
// gbqrf: one group (one warp, or the whole CTA for wide bands) walks the columns.
// The active part at step k is the (l+1) x (u+1) window A(k:k+l, k:k+u) (u already
// includes the l padding bands _banded_qr adds, bandedqr.jl:2); it is kept in shared
// memory as a ring in both dimensions, exactly like the LU window, and the row
// entering at each step is prefetched with cp.async.  Per step:
//   * warp 0 forms the reflector of column k as LinearAlgebra.reflector! does
//     (2-norm, nu = copysign(norm, x1), x1 <- -nu, x_i <- x_i / (x1 + nu),
//     tau = (x1 + nu) / nu), the divisions spread over the group.  The norm is the
//     one a SIMD BLAS nrm2 forms: max|x| first; squares of x itself when max|x| lies
//     in [2^-400, 2^400] (f32: [2^-50, 2^50]), else of x / max|x|, summed in four
//     interleaved fma partial sums combined as (s0 + s1) + (s2 + s3);
//   * every following column of the window is shared by four threads, which apply the
//     reflector as reflectorApply! does: v = tau * (a_0 + x'a) with the dot product in
//     the same four-way interleaved order, a_0 -= v, a_i = fma(-v, x_i, a_i).
// The results equal the oracle's restatement bit for bit.
//
// gbqr_lmul: Q or Q' times B, one thread per right-hand side column running the
// reference loop (sequential fma dot products, so again bit for bit).
#include "lu.cuh"
#include "tri.cuh"

namespace bm {

// Column stride of the QR window: >= l+1 and 4 (mod 32).  A warp's reflector
// application reads eight columns with four threads each (rows r+sub, sub = 0..3), so
// the column offsets 4c keep the 32 threads on distinct banks for 32-bit elements and
// the 16 threads of each half-warp on distinct bank pairs for 64-bit ones.
__host__ __device__ inline int qr_rs(int l) { return ((l + 1 + 27) & ~31) + 4; }
template <int P>
__host__ __device__ inline i64 gbqrf_smem_elems(int l, int u) {
  const int K = u + 1;
  return kHdr + (i64)qr_rs(l) * K + (i64)P * K + (l + 1);  // header + window + staging ring
}

template <typename T, int P, int G>
__device__ void gbqrf_group(i64 m, i64 n, int l, int u, T* __restrict__ D, i64 ldd, T* __restrict__ tau,
                            T* __restrict__ smem) {
  constexpr int NT = Grp<G>::NT;
  const int tid = Grp<G>::tid();
  const int R = l + 1, K = u + 1, RS = qr_rs(l);
  T* hdr = smem;  // hdr[0] = tau_k, hdr[1] = xi1 (x1 + nu)
  T* W = smem + kHdr;
  T* S = W + (i64)RS * K;
  const i64 ncols = min(m - 1, n);
  for (i64 e = tid; e < min(m, n); e += NT) tau[e] = T(0);
  if (ncols <= 0) return;

  // initial window: matrix rows 0..l, columns 0..u (D(i,c) = D[(u + i - c) + c*ldd])
  for (int e = tid; e < R * K; e += NT) {
    const int c = e / R, r = e - c * R;
    T v = T(0);
    if (r < m && c < n && r - c <= l && c - r <= u) v = D[(u + r - c) + (i64)c * ldd];
    W[r + c * RS] = v;
  }
  auto issue_row = [&](i64 i) {
    T* dst = S + (int)(i & (P - 1)) * K;
    for (int c = tid; c < K; c += NT) {
      const i64 col = i - l + c;
      const bool ok = i < m && col < n;
      cp_async_elem(dst + c, ok ? D + (u + l - c) + col * ldd : D, ok);
    }
    cp_async_commit();
  };
  for (int p = 0; p < P; ++p) issue_row((i64)l + 1 + p);
  Grp<G>::sync();

  int pr0 = 0, pc0 = 0;
  for (i64 k = 0; k < ncols; ++k) {
    const int len = (int)min((i64)(l + 1), m - k);  // reflector length
    T* x = W + pc0 * RS;                             // logical column 0 (ring rows)
    auto prow = [&](int r) {
      int pr = pr0 + r;
      return pr >= R ? pr - R : pr;
    };
    // ---- reflector (warp 0).  max|x| through integer keys; the sum of squares in four
    // interleaved partial sums (lane t takes rows t, t+4, ...), combined (s0+s1)+(s2+s3);
    // squares taken directly when max|x| is in a safe range, else of x/max|x|.
    if (tid < 32) {
      const int lane = tid;
      unsigned long long key = 0ull;
      for (int i = lane; i < len; i += 32) {
        const unsigned long long kk = pivot_key(x[prow(i)], false);  // NaN never raises the scale
        key = kk > key ? kk : key;
      }
      const unsigned mhi = __reduce_max_sync(0xffffffffu, (unsigned)(key >> 32));
      const unsigned mlo = __reduce_max_sync(0xffffffffu, (unsigned)(key >> 32) == mhi ? (unsigned)key : 0u);
      const unsigned long long mkey = ((unsigned long long)mhi << 32) | mlo;
      T scale;
      if constexpr (sizeof(T) == 8) scale = __longlong_as_double((long long)mkey);
      else scale = __uint_as_float((unsigned)mkey);
      const bool finite_nz = scale != T(0) && isfinite(scale);
      const bool direct = sizeof(T) == 8 ? (scale > T(0x1p-400) && scale < T(0x1p400))
                                         : (scale > T(0x1p-50) && scale < T(0x1p50));
      T part = T(0);
      if (finite_nz && lane < 4)
        for (int i = lane; i < len; i += 4) {
          const T t = direct ? x[prow(i)] : x[prow(i)] / scale;
          part = fma(t, t, part);
        }
      part += __shfl_xor_sync(0xffffffffu, part, 1);
      part += __shfl_xor_sync(0xffffffffu, part, 2);
      T tk = T(0), xi1 = T(0);
      if (lane == 0) {
        if (scale != T(0)) {
          const T normu = !finite_nz ? scale : (direct ? sqrt(part) : scale * sqrt(part));
          const T x1 = x[pr0];
          const T nu = copysign(normu, x1);
          xi1 = x1 + nu;
          x[pr0] = -nu;
          tk = xi1 / nu;
        }
        hdr[0] = tk;
        tau[k] = tk;
      }
      tk = __shfl_sync(0xffffffffu, tk, 0);
      xi1 = __shfl_sync(0xffffffffu, xi1, 0);
      // the reflector x(2:len) / (x1 + nu), final: to the factor storage, with R(k,k)
      if (xi1 != T(0) || tk != T(0))
        for (int i = 1 + lane; i < len; i += 32) x[prow(i)] = x[prow(i)] / xi1;
      __syncwarp();
      for (int r = lane; r < len; r += 32) D[(u + r) + k * ldd] = x[prow(r)];
    }
    Grp<G>::sync();
    const T tk = hdr[0];
    // ---- apply to columns k+1 .. k+min(u, n-1-k): four threads per column, the dot
    // product in four interleaved partial sums (rows 1+t, 5+t, ...) combined
    // (s0+s1)+(s2+s3), then each thread updates its own rows; row k of R is final and
    // goes to the factor storage
    const int nc = (int)min((i64)u, n - 1 - k);
    const int sub = tid & 3;
    for (int base = 0; base < nc; base += NT / 4) {
      const int c = 1 + base + (tid >> 2);
      const bool act = c <= nc;
      int pc = pc0 + c;
      pc = pc >= K ? pc - K : pc;
      T* a = W + (act ? pc : pc0) * RS;
      const T a0 = act ? a[pr0] : T(0);
      T part = T(0);
      if (act)
        for (int i = 1 + sub; i < len; i += 4) part = fma(x[prow(i)], a[prow(i)], part);
      part += __shfl_xor_sync(0xffffffffu, part, 1);
      part += __shfl_xor_sync(0xffffffffu, part, 2);
      if (act) {
        const T v = tk * (a0 + part);
        if (sub == 0) {
          a[pr0] = a0 - v;
          D[(u - c) + (k + c) * ldd] = a0 - v;
        }
        for (int i = 1 + sub; i < len; i += 4) a[prow(i)] = fma(-v, x[prow(i)], a[prow(i)]);
      }
    }
    if (k + 1 == ncols) break;
    Grp<G>::sync();  // every read of column k and row k is done
    // ---- slide: row k+1+l enters physical row pr0, column k+1+u enters physical column
    // pc0 (zero above the entering row).  A thread stores the staged entries it copied
    // itself, so its own wait is enough; the zeroing leaves row pr0 to the entering row.
    for (int r = tid; r < R; r += NT)
      if (r != pr0) W[r + pc0 * RS] = T(0);
    cp_async_wait<P - 1>();
    const i64 inew = k + 1 + l;
    const T* st = S + (int)(inew & (P - 1)) * K;
    for (int c = tid; c < K; c += NT) {
      int pc = pc0 + 1 + c;
      pc = pc >= K ? pc - K : pc;
      W[pr0 + pc * RS] = st[c];
    }
    Grp<G>::sync();
    issue_row(inew + P);
    pr0 = pr0 + 1 == R ? 0 : pr0 + 1;
    pc0 = pc0 + 1 == K ? 0 : pc0 + 1;
  }
  cp_async_wait<0>();
  Grp<G>::sync();
  // rows ncols.. of R that the loop never slid out (m <= n: the last row; the window
  // still holds final values for rows k+1 .. k+l and their columns)
  {
    const i64 k = ncols - 1;
    for (int e = tid; e < R * K; e += NT) {
      const int c = e / R, r = e - c * R;
      if (r == 0) continue;  // row k was written above
      const i64 i = k + r, col = k + c;
      if (i < m && col < n && col >= i && col - i <= u) {
        int pr = pr0 + r;
        pr = pr >= R ? pr - R : pr;
        int pc = pc0 + c;
        pc = pc >= K ? pc - K : pc;
        D[(u + i - col) + col * ldd] = W[pr + pc * RS];
      }
    }
  }
  Grp<G>::sync();
}

template <typename T, int G>
__global__ void __launch_bounds__(32 * G) gbqrf_kernel(i64 m, i64 n, int l, int u, T* D, i64 ldd, T* tau) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  gbqrf_group<T, 4, G>(m, n, l, u, D, ldd, tau, reinterpret_cast<T*>(smem_raw));
}

// Q*B (adjoint = false) or Q'*B (adjoint = true): thread c owns column c of B.
template <typename T>
__global__ void gbqr_lmul_kernel(bool adjoint, i64 m, i64 n, int l, int u, const T* __restrict__ D, i64 ldd,
                                 const T* __restrict__ tau, i64 ntau, i64 nrhs, T* __restrict__ B, i64 ldb) {
  // four threads per right-hand side: thread q takes rows k+1+q, k+5+q, ... of each
  // reflector, so the dot product has the four interleaved partial sums of gbqrf's
  // reflector application, combined (s0+s1)+(s2+s3) by two butterfly shuffles
  const i64 c = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 2;
  const int q = threadIdx.x & 3;
  const bool live = c < nrhs;
  T* b = B + (live ? c : 0) * ldb;
  const i64 kmax = min(min(m, n), ntau);
  const int ilo = max(1, -u);
  for (i64 t = 0; t < kmax; ++t) {
    const i64 k = adjoint ? t : kmax - 1 - t;
    const T* d = D + (u - k) + k * ldd;  // d[i] = D[(i - k + u), k]
    const i64 ihi = min(k + l, m - 1);
    T part = T(0);
    if (live)
      for (i64 i = k + 1 + q; i <= ihi; i += 4)
        if (i >= k + ilo) part = fma(d[i], b[i], part);
    part += __shfl_xor_sync(0xffffffffu, part, 1);
    part += __shfl_xor_sync(0xffffffffu, part, 2);
    if (live) {
      const T bk = b[k];
      const T v = tau[k] * (bk + part);
      for (i64 i = k + 1 + q; i <= ihi; i += 4)
        if (i >= k + ilo) b[i] = fma(-d[i], v, b[i]);
      __syncwarp(0xfu << (threadIdx.x & 28));  // the group's reads of b[k] precede the store
      if (q == 0) b[k] = bk - v;
    }
    __syncwarp();
  }
}

// Upper triangular band solve (tbsv 'U', non-unit): the gbtrs sweeps with kl = 0.
template <typename T, int G>
__global__ void __launch_bounds__(32 * G) tbsv_upper_kernel(bool trans, i64 n, int k, const T* A, i64 lda, T* x,
                                                            i64 ldx, i64 nrhs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  for (i64 r = blockIdx.x; r * kMaxRhs < nrhs; r += gridDim.x)
    gbtrs_all<T, G>(trans, n, 0, k, min((i64)kMaxRhs, nrhs - r * kMaxRhs), A, lda, nullptr, x + r * kMaxRhs * ldx,
                    ldx, reinterpret_cast<T*>(smem_raw));
}

template <typename T>
static int gbqrf_impl(i64 m, i64 n, i64 l, i64 u, T* D, i64 ldd, T* tau, cudaStream_t stream, const char* name) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (l < 0) return -3;
  if (u < 0) return -4;
  if (ldd < l + u + 1) return -6;
  if (m == 0 || n == 0) return BM_OK;
  if (!tau) return -7;
  const i64 bytes = gbqrf_smem_elems<4>((int)l, (int)u) * (i64)sizeof(T);
  if (bytes > 227 * 1024) {
    set_error("%s: band (l=%lld, u=%lld) exceeds the window limit", name, (long long)l, (long long)u);
    return BM_ERR_UNSUPPORTED;
  }
  if (u >= 48) {  // four threads per following column: 8 warps cover 64 columns per pass
    int r = cuda_status(ensure_smem((const void*)gbqrf_kernel<T, 8>, (int)bytes), name);
    if (r) return r;
    gbqrf_kernel<T, 8><<<1, 256, (int)bytes, stream>>>(m, n, (int)l, (int)u, D, ldd, tau);
  } else if ((l + 1) * (u + 1) >= 512) {
    int r = cuda_status(ensure_smem((const void*)gbqrf_kernel<T, 4>, (int)bytes), name);
    if (r) return r;
    gbqrf_kernel<T, 4><<<1, 128, (int)bytes, stream>>>(m, n, (int)l, (int)u, D, ldd, tau);
  } else {
    int r = cuda_status(ensure_smem((const void*)gbqrf_kernel<T, 1>, (int)bytes), name);
    if (r) return r;
    gbqrf_kernel<T, 1><<<1, 32, (int)bytes, stream>>>(m, n, (int)l, (int)u, D, ldd, tau);
  }
  return launch_status(name);
}

template <typename T>
static int gbqr_lmul_impl(char trans, i64 m, i64 n, i64 l, i64 u, const T* D, i64 ldd, const T* tau, i64 ntau,
                          i64 nrhs, T* B, i64 ldb, cudaStream_t stream, const char* name) {
  const bool adj = (trans == 'T' || trans == 't' || trans == 'C' || trans == 'c');
  if (!adj && !(trans == 'N' || trans == 'n')) return -1;
  if (m < 0) return -2;
  if (n < 0) return -3;
  if (l < 0) return -4;
  if (ldd < l + std::max<i64>(u, 0) + 1) return -7;
  if (ntau < 0) return -9;
  if (nrhs < 0) return -10;
  if (ldb < std::max<i64>(1, m)) return -12;
  if (m == 0 || nrhs == 0 || ntau == 0) return BM_OK;
  const int threads = nrhs <= 8 ? 32 : 128;  // whole warps: four lanes per right-hand side
  gbqr_lmul_kernel<T><<<(unsigned)ceil_div(4 * nrhs, threads), threads, 0, stream>>>(adj, m, n, (int)l, (int)u, D,
                                                                                      ldd, tau, ntau, nrhs, B, ldb);
  return launch_status(name);
}

template <typename T>
static int tbsv_impl(char uplo, char trans, char diag, i64 n, i64 k, const T* A, i64 lda, T* x, i64 incx,
                     cudaStream_t stream, const char* name) {
  const bool upper = (uplo == 'U' || uplo == 'u');
  if (!upper && !(uplo == 'L' || uplo == 'l')) return -1;
  const bool tr = (trans == 'T' || trans == 't' || trans == 'C' || trans == 'c');
  if (!tr && !(trans == 'N' || trans == 'n')) return -2;
  if (!(diag == 'N' || diag == 'n' || diag == 'U' || diag == 'u')) return -3;
  if (n < 0) return -4;
  if (k < 0) return -5;
  if (lda < k + 1) return -7;
  if (incx == 0) return -9;
  if (n == 0) return BM_OK;
  // lower, unit-diagonal or strided forms: the general one-warp sweep (tri.cu)
  if (!upper || diag == 'U' || diag == 'u' || incx != 1)
    return tbsv_general<T>(uplo, trans, diag, n, k, A, lda, x, incx, stream, name);
  const i64 bytes = gbtrs_smem_elems(0, (int)k) * (i64)sizeof(T);
  if (bytes > 227 * 1024) {
    set_error("%s: band too wide for the staged solve", name);
    return BM_ERR_UNSUPPORTED;
  }
  int r = cuda_status(ensure_smem((const void*)tbsv_upper_kernel<T, 4>, (int)bytes), name);
  if (r) return r;
  tbsv_upper_kernel<T, 4><<<1, 128, (int)bytes, stream>>>(tr, n, (int)k, A, lda, x, std::max<i64>(1, n), 1);
  return launch_status(name);
}

}  // namespace bm

extern "C" int bm_dgbqrf(int64_t m, int64_t n, int64_t l, int64_t u, double* AB, int64_t ldab, double* tau,
                         bm_stream_t stream) {
  return bm::gbqrf_impl<double>(m, n, l, u, AB, ldab, tau, reinterpret_cast<cudaStream_t>(stream), "bm_dgbqrf");
}
extern "C" int bm_sgbqrf(int64_t m, int64_t n, int64_t l, int64_t u, float* AB, int64_t ldab, float* tau,
                         bm_stream_t stream) {
  return bm::gbqrf_impl<float>(m, n, l, u, AB, ldab, tau, reinterpret_cast<cudaStream_t>(stream), "bm_sgbqrf");
}
extern "C" int bm_dgbqr_lmul(char trans, int64_t m, int64_t n, int64_t l, int64_t u, const double* AB, int64_t ldab,
                             const double* tau, int64_t ntau, int64_t nrhs, double* B, int64_t ldb,
                             bm_stream_t stream) {
  return bm::gbqr_lmul_impl<double>(trans, m, n, l, u, AB, ldab, tau, ntau, nrhs, B, ldb,
                                    reinterpret_cast<cudaStream_t>(stream), "bm_dgbqr_lmul");
}
extern "C" int bm_sgbqr_lmul(char trans, int64_t m, int64_t n, int64_t l, int64_t u, const float* AB, int64_t ldab,
                             const float* tau, int64_t ntau, int64_t nrhs, float* B, int64_t ldb, bm_stream_t stream) {
  return bm::gbqr_lmul_impl<float>(trans, m, n, l, u, AB, ldab, tau, ntau, nrhs, B, ldb,
                                   reinterpret_cast<cudaStream_t>(stream), "bm_sgbqr_lmul");
}
extern "C" int bm_dtbsv(char uplo, char trans, char diag, int64_t n, int64_t k, const double* A, int64_t lda, double* x,
                        int64_t incx, bm_stream_t stream) {
  return bm::tbsv_impl<double>(uplo, trans, diag, n, k, A, lda, x, incx, reinterpret_cast<cudaStream_t>(stream),
                               "bm_dtbsv");
}
extern "C" int bm_stbsv(char uplo, char trans, char diag, int64_t n, int64_t k, const float* A, int64_t lda, float* x,
                        int64_t incx, bm_stream_t stream) {
  return bm::tbsv_impl<float>(uplo, trans, diag, n, k, A, lda, x, incx, reinterpret_cast<cudaStream_t>(stream),
                              "bm_stbsv");
}
