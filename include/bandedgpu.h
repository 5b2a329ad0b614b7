/*
 * bandedgpu -- C ABI of the GB300 (sm_103a) banded linear-algebra library.
 *
 * Drop-in replacement for the native calls BandedMatrices.jl makes on its
 * banded hot path.  Every routine:
 *   - takes DEVICE pointers (column-major, LAPACK band storage) and an explicit
 *     cudaStream_t (pass 0 for the legacy default stream);
 *   - only enqueues work on that stream: no host synchronisation;
 *   - returns BM_OK, or -i when argument i is illegal (LAPACK convention,
 *     arguments numbered from 1), or a BM_ERR_* code;
 *   - writes numerical status (LAPACK `info`) to device memory.
 * Integers are int64_t (Julia's BlasInt on ILP64 builds); pivot vectors are
 * int64_t and 1-based, as LAPACK and BandedLU.ipiv store them.
 *
 * Band storage: a BandedMatrix with bandwidths (l,u) keeps its entries in a
 * (l+u+1) x n column-major array with A[k,j] = data[u+k-j, j] (0-based;
 * src/banded/BandedMatrix.jl:16-28, :414-419).  The LU factors use the
 * (2l+u+1) x n gbtrf layout (src/banded/BandedLU.jl:108-111).
 */
#ifndef BANDEDGPU_H
#define BANDEDGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *bm_stream_t; /* identical to cudaStream_t */

enum {
  BM_OK = 0,
  BM_ERR_CUDA = -1001,        /* a CUDA call failed; see bm_last_error() */
  BM_ERR_UNSUPPORTED = -1002, /* valid arguments this build does not handle */
  BM_ERR_NOMEM = -1003,       /* workspace allocation failed */
  BM_ERR_ALIGN = -1004        /* a pointer lacks the alignment the routine needs */
};

/* Library version (major*10000 + minor*100 + patch). */
int bm_version(void);

/* Text of the last error raised on the calling host thread ("" if none). */
const char *bm_last_error(void);

/* Device status word of the current device: bit 0 is set when a bounded
 * in-kernel wait expired.  `clear` resets it.  Synchronises the stream. */
int bm_device_status(int *status_out, int clear, bm_stream_t stream);

/* ------------------------------------------------------------------ gbmv
 * y <- alpha*op(A)*x + beta*y, op = 'N' | 'T' (| 'C' = 'T' for real types).
 * Replaces the dgbmv_/sgbmv_ ccall of src/blas.jl:16-28 and the stdlib
 * BLAS.gbmv! call of banded_gbmv! (src/generic/matmul.jl:21-23) reached from
 * A*x / mul!(y,A,x,alpha,beta) (materialize!, src/generic/matmul.jl:61-92).
 * Argument order and meaning are those of BLAS xGBMV.  beta == 0 means y is
 * not read (NaN in y is overwritten), as in reference BLAS. */
int bm_dgbmv(char trans, int64_t m, int64_t n, int64_t kl, int64_t ku, double alpha, const double *A,
             int64_t lda, const double *x, int64_t incx, double beta, double *y, int64_t incy,
             bm_stream_t stream);
int bm_sgbmv(char trans, int64_t m, int64_t n, int64_t kl, int64_t ku, float alpha, const float *A,
             int64_t lda, const float *x, int64_t incx, float beta, float *y, int64_t incy,
             bm_stream_t stream);

/* ------------------------------------------------------------------ gbmm
 * C <- alpha*A*B + beta*C for banded A (n x nu, bandwidths (Al,Au)), B (nu x m,
 * (Bl,Bu)) and C (n x m, (Cl,Cu)), all bandwidths >= 0 and C's band wide enough
 * for every in-matrix nonzero of A*B: Cl >= min(Al+Bl, n-1), Cu >= min(Au+Bu, m-1).
 * Bands of C beyond the product are scaled by beta; beta == 0 means C is not read.
 * Replaces gbmm!/_gbmm! (src/banded/gbmm.jl:207-340), reached from A*B and
 * mul!(C,A,B,alpha,beta) (materialize!, src/generic/matmul.jl:177-189); each C
 * entry equals the column dgbmv of _gbmm! bit for bit. */
int bm_dgbmm(int64_t n, int64_t nu, int64_t m, int64_t Al, int64_t Au, int64_t Bl, int64_t Bu, int64_t Cl,
             int64_t Cu, double alpha, const double *A, int64_t lda, const double *B, int64_t ldb, double beta,
             double *C, int64_t ldc, bm_stream_t stream);
int bm_sgbmm(int64_t n, int64_t nu, int64_t m, int64_t Al, int64_t Au, int64_t Bl, int64_t Bu, int64_t Cl,
             int64_t Cu, float alpha, const float *A, int64_t lda, const float *B, int64_t ldb, float beta,
             float *C, int64_t ldc, bm_stream_t stream);

/* flags[r] <- 1 if band r (storage row r) of the m x n band matrix (l,u) holds a
 * nonzero in-matrix entry, else 0 (flags: l+u+1 device ints).  The device side of
 * _num_zeroband_u/_num_zeroband_l (src/banded/gbmm.jl:191-205), which gbmm! uses
 * to accept a C narrower than the product. */
int bm_dgb_nonzero_bands(int64_t m, int64_t n, int64_t l, int64_t u, const double *A, int64_t lda, int *flags,
                         bm_stream_t stream);
int bm_sgb_nonzero_bands(int64_t m, int64_t n, int64_t l, int64_t u, const float *A, int64_t lda, int *flags,
                         bm_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* BANDEDGPU_H */
