// Triangular band solve and product: xTBSV (x <- op(A)^-1 x) and xTBMV (x <- op(A) x)
// for a triangular band A (k super- or sub-diagonals) in BLAS triangular band storage,
// every uplo / trans / diag form and any nonzero incx.
//
// Replaces the tbsv!/tbmv! ccalls of src/blas.jl:71-147, reached from
// UpperTriangular/LowerTriangular(::BandedMatrix) \ x and * x (src/tribanded.jl:47-96).
// Each element receives the operations of reference BLAS DTBSV / DTBMV in their order,
// with every multiply-add fused, so the results equal the oracle's bit for bit.
//
// tbsv is a chain of n dependent steps; one warp sweeps it.  The axpy forms ('N')
// finish x(j) (divided by the diagonal unless unit, skipped when x(j) == 0, as DTBSV
// does) and hand the k elements it reaches to the lanes; the dot forms ('T') load the
// window's k terms across the lanes and run the sum in DTBSV's order on every lane.
//
// tbmv is a product: every output depends only on the input vector.  One CTA sweeps
// tiles of 256 outputs in the direction that never reads an element after a tile has
// overwritten it (the 'ahead' forms -- N/U and T/L read x(i .. i+k) -- ascending,
// the others descending); inside a tile every thread computes its output from the old
// values, the CTA synchronises, then the tile is written.
#include "tri.cuh"

namespace bm {

template <typename T>
struct StridedVec {
  T* p;
  i64 inc, kx;  // logical element j at p[kx + j * inc] (BLAS convention for negative inc)
  __device__ __forceinline__ T& operator[](i64 j) const { return p[kx + j * inc]; }
};

template <typename T>
__device__ void tbsv_warp(bool upper, bool trans, bool unit, i64 n, int k, const T* __restrict__ A, i64 lda, T* x,
                          i64 incx) {
  const int lane = threadIdx.x & 31;
  const StridedVec<T> X{x, incx, incx > 0 ? 0 : -(n - 1) * incx};
  if (!trans) {
    for (i64 s = 0; s < n; ++s) {
      const i64 j = upper ? n - 1 - s : s;
      T xj = X[j];
      if (xj != T(0)) {
        if (!unit) xj = xj / A[(upper ? k : 0) + j * lda];
        const T temp = -xj;
        if (upper) {
          const i64 lo = max((i64)0, j - k);
          for (i64 i = j - 1 - lane; i >= lo; i -= 32) X[i] = fma(temp, A[(k - j + i) + j * lda], X[i]);
        } else {
          const i64 hi = min(n - 1, j + k);
          for (i64 i = j + 1 + lane; i <= hi; i += 32) X[i] = fma(temp, A[(i - j) + j * lda], X[i]);
        }
        if (lane == 0) X[j] = xj;
      }
      __syncwarp();
    }
  } else {
    for (i64 s = 0; s < n; ++s) {
      const i64 j = upper ? s : n - 1 - s;
      T temp = X[j];
      // terms in DTBSV's order: upper i = j-k .. j-1 ascending, lower i = j+k .. j+1 descending
      const i64 cnt = upper ? j - max((i64)0, j - k) : min(n - 1, j + k) - j;
      for (i64 q0 = 0; q0 < cnt; q0 += 32) {
        const i64 q = q0 + lane;
        T na = T(0), xv = T(0);
        if (q < cnt) {
          const i64 i = upper ? max((i64)0, j - k) + q : min(n - 1, j + k) - q;
          na = -A[(upper ? k - j + i : i - j) + j * lda];
          xv = X[i];
        }
        const int m = (int)min((i64)32, cnt - q0);
        for (int t = 0; t < m; ++t) temp = fma(__shfl_sync(0xffffffffu, na, t), __shfl_sync(0xffffffffu, xv, t), temp);
      }
      if (!unit) temp = temp / A[(upper ? k : 0) + j * lda];
      __syncwarp();
      if (lane == 0) X[j] = temp;
      __syncwarp();
    }
  }
}

// Vector v = blockIdx.x (grid-stride) of nvec, at x + v * ldx.
template <typename T>
__global__ void __launch_bounds__(32) tbsv_warp_kernel(bool upper, bool trans, bool unit, i64 n, int k,
                                                       const T* __restrict__ A, i64 lda, T* x, i64 incx, i64 nvec,
                                                       i64 ldx) {
  for (i64 v = blockIdx.x; v < nvec; v += gridDim.x) tbsv_warp(upper, trans, unit, n, k, A, lda, x + v * ldx, incx);
}

constexpr int kTbmvThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kTbmvThreads) tbmv_tile_kernel(bool upper, bool trans, bool unit, i64 n, int k,
                                                                 const T* __restrict__ A, i64 lda, T* x, i64 incx) {
  const StridedVec<T> X{x, incx, incx > 0 ? 0 : -(n - 1) * incx};
  const bool ahead = upper != trans;  // N/U and T/L read x(i .. i+k)
  const i64 ntiles = (n + kTbmvThreads - 1) / kTbmvThreads;
  for (i64 t = 0; t < ntiles; ++t) {
    const i64 tile = ahead ? t : ntiles - 1 - t;
    const i64 i = tile * kTbmvThreads + threadIdx.x;
    T acc = T(0);
    if (i < n) {
      if (!trans) {  // DTBMV 'N': x(i) scaled by its diagonal at step i, then the column updates
        const T xi = X[i];
        acc = (xi != T(0) && !unit) ? xi * A[(upper ? k : 0) + i * lda] : xi;
        if (upper) {
          const i64 hi = min(n - 1, i + k);
          for (i64 j = i + 1; j <= hi; ++j) {
            const T xj = X[j];
            if (xj != T(0)) acc = fma(xj, A[(k + i - j) + j * lda], acc);
          }
        } else {
          const i64 lo = max((i64)0, i - k);
          for (i64 j = i - 1; j >= lo; --j) {
            const T xj = X[j];
            if (xj != T(0)) acc = fma(xj, A[(i - j) + j * lda], acc);
          }
        }
      } else {  // DTBMV 'T': the dot product of column i with x, diagonal first
        acc = X[i];
        if (!unit) acc = acc * A[(upper ? k : 0) + i * lda];
        if (upper) {
          const i64 lo = max((i64)0, i - k);
          for (i64 r = i - 1; r >= lo; --r) acc = fma(A[(k + r - i) + i * lda], X[r], acc);
        } else {
          const i64 hi = min(n - 1, i + k);
          for (i64 r = i + 1; r <= hi; ++r) acc = fma(A[(r - i) + i * lda], X[r], acc);
        }
      }
    }
    __syncthreads();
    if (i < n) X[i] = acc;
    __syncthreads();
  }
}

// Argument checks of xTBSV / xTBMV (BLAS numbering: uplo 1, trans 2, diag 3, n 4, k 5,
// lda 7, incx 9); 0 when legal.
static int tri_check(char uplo, char trans, char diag, i64 n, i64 k, i64 lda, i64 incx) {
  if (!(uplo == 'U' || uplo == 'u' || uplo == 'L' || uplo == 'l')) return -1;
  if (!(trans == 'N' || trans == 'n' || trans == 'T' || trans == 't' || trans == 'C' || trans == 'c')) return -2;
  if (!(diag == 'N' || diag == 'n' || diag == 'U' || diag == 'u')) return -3;
  if (n < 0) return -4;
  if (k < 0) return -5;
  if (lda < k + 1) return -7;
  if (incx == 0) return -9;
  return 0;
}

template <typename T>
int tbsv_general(char uplo, char trans, char diag, i64 n, i64 k, const T* A, i64 lda, T* x, i64 incx,
                 cudaStream_t stream, const char* name, i64 nvec, i64 ldx) {
  if (int r = tri_check(uplo, trans, diag, n, k, lda, incx)) return r;
  if (n == 0 || nvec == 0) return BM_OK;
  if (k > 0x7fffffff) return -5;
  const i64 grid = std::min<i64>(nvec, (i64)num_sms() * 16);
  tbsv_warp_kernel<T><<<(unsigned)grid, 32, 0, stream>>>(uplo == 'U' || uplo == 'u', !(trans == 'N' || trans == 'n'),
                                                         diag == 'U' || diag == 'u', n, (int)k, A, lda, x, incx, nvec,
                                                         ldx);
  return launch_status(name);
}
template int tbsv_general<double>(char, char, char, i64, i64, const double*, i64, double*, i64, cudaStream_t,
                                  const char*, i64, i64);
template int tbsv_general<float>(char, char, char, i64, i64, const float*, i64, float*, i64, cudaStream_t,
                                 const char*, i64, i64);

template <typename T>
static int tbmv_impl(char uplo, char trans, char diag, i64 n, i64 k, const T* A, i64 lda, T* x, i64 incx,
                     cudaStream_t stream, const char* name) {
  if (int r = tri_check(uplo, trans, diag, n, k, lda, incx)) return r;
  if (n == 0) return BM_OK;
  if (k > 0x7fffffff) return -5;
  tbmv_tile_kernel<T><<<1, kTbmvThreads, 0, stream>>>(uplo == 'U' || uplo == 'u', !(trans == 'N' || trans == 'n'),
                                                      diag == 'U' || diag == 'u', n, (int)k, A, lda, x, incx);
  return launch_status(name);
}

}  // namespace bm

extern "C" int bm_dtbmv(char uplo, char trans, char diag, int64_t n, int64_t k, const double* A, int64_t lda,
                        double* x, int64_t incx, bm_stream_t stream) {
  return bm::tbmv_impl<double>(uplo, trans, diag, n, k, A, lda, x, incx, reinterpret_cast<cudaStream_t>(stream),
                               "bm_dtbmv");
}
extern "C" int bm_stbmv(char uplo, char trans, char diag, int64_t n, int64_t k, const float* A, int64_t lda, float* x,
                        int64_t incx, bm_stream_t stream) {
  return bm::tbmv_impl<float>(uplo, trans, diag, n, k, A, lda, x, incx, reinterpret_cast<cudaStream_t>(stream),
                              "bm_stbmv");
}
