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

/* Diagnostics (no reference counterpart).  Kernels this library has enqueued in
 * the process, captured launches included. */
unsigned long long bm_launch_count(void);

/* The fma rate (fmas per second) the current GPU sustains for elements of
 * elem_bytes = 8 (Float64) or 4 (Float32): the compute roof of the kernels the
 * FP64 pipe bounds.  Runs a short probe kernel; synchronises the stream. */
int bm_probe_fma_rate(int elem_bytes, double *fma_per_s, bm_stream_t stream);

/* Diagnostics (no reference counterpart).  Self-test of the bounded in-kernel waits:
 * enqueues a one-thread kernel that waits, with the same helper the streaming kernels
 * use, for an mbarrier phase that nothing completes, giving up after spin_limit polls
 * (1 <= spin_limit <= 2^26).  On expiry the kernel sets bit 0 (timeout) of the device
 * status word (read it with bm_device_status) and returns; *done (device int) is set
 * to 1 once the wait has ended.  Nothing faults, traps or hangs. */
int bm_wait_selftest(int64_t spin_limit, int *done, bm_stream_t stream);

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

/* ------------------------------------------------------------------ LU
 * Partial-pivot banded LU, LAPACK xGBTRF: AB is the (2kl+ku+1) x n gbtrf storage
 * (ldab >= 2kl+ku+1; matrix in rows kl..2kl+ku, the top kl rows receive fill-in),
 * factored in place; ipiv receives min(m,n) 1-based pivots; *info (device) receives
 * LAPACK's info (0, or i > 0 when U(i,i) is exactly zero).  Factors and pivots equal
 * unblocked dgbtf2's bit for bit.  Replaces LAPACK.gbtrf! in lu!
 * (src/banded/BandedLU.jl:90-103), which BandedMatrices.jl calls as
 * gbtrf!(l, u-l, m, data) on the band re-widened to (l, l+u) by _lu (:108-111). */
int bm_dgbtrf(int64_t m, int64_t n, int64_t kl, int64_t ku, double *AB, int64_t ldab, int64_t *ipiv, int64_t *info,
              bm_stream_t stream);
int bm_sgbtrf(int64_t m, int64_t n, int64_t kl, int64_t ku, float *AB, int64_t ldab, int64_t *ipiv, int64_t *info,
              bm_stream_t stream);

/* Solve op(A) X = B with the xGBTRF factors, LAPACK xGBTRS (trans 'N' or 'T'/'C');
 * B is n x nrhs column-major (ldb >= max(1,n)), overwritten with X.  Replaces
 * LAPACK.gbtrs! in ldiv!(::BandedLU, B) (src/banded/linalg.jl:24-30) and
 * ldiv!(transpose(F), B) (:41-47, :55-56). */
int bm_dgbtrs(char trans, int64_t n, int64_t kl, int64_t ku, int64_t nrhs, const double *AB, int64_t ldab,
              const int64_t *ipiv, double *B, int64_t ldb, bm_stream_t stream);
int bm_sgbtrs(char trans, int64_t n, int64_t kl, int64_t ku, int64_t nrhs, const float *AB, int64_t ldab,
              const int64_t *ipiv, float *B, int64_t ldb, bm_stream_t stream);

/* ------------------------------------------------------------------ QR
 * Householder QR of the m x n band in AB, in place: AB holds the matrix with
 * bandwidths (l, u) where u already includes the l extra bands that receive the
 * fill of R (qr(A) widens A from (l, u0) to (l, l+u0), src/banded/bandedqr.jl:1-2);
 * ldab >= l+u+1.  On exit the upper band holds R and the l rows below the diagonal
 * hold the reflectors; tau (min(m,n) entries) receives their scalars, zero beyond
 * min(m-1,n).  Reflector convention of LinearAlgebra.reflector!.  Replaces
 * _banded_qr! (src/banded/bandedqr.jl:13-28). */
int bm_dgbqrf(int64_t m, int64_t n, int64_t l, int64_t u, double *AB, int64_t ldab, double *tau,
              bm_stream_t stream);
int bm_sgbqrf(int64_t m, int64_t n, int64_t l, int64_t u, float *AB, int64_t ldab, float *tau, bm_stream_t stream);

/* B <- Q*B (trans 'N') or Q'*B ('T'/'C') with the bm_*gbqrf factors (m x n,
 * bandwidths (l,u), ntau reflectors); B is m x nrhs, leading dim ldb.  Replaces
 * banded_qr_lmul! (src/banded/bandedqr.jl:38-94). */
int bm_dgbqr_lmul(char trans, int64_t m, int64_t n, int64_t l, int64_t u, const double *AB, int64_t ldab,
                  const double *tau, int64_t ntau, int64_t nrhs, double *B, int64_t ldb, bm_stream_t stream);
int bm_sgbqr_lmul(char trans, int64_t m, int64_t n, int64_t l, int64_t u, const float *AB, int64_t ldab,
                  const float *tau, int64_t ntau, int64_t nrhs, float *B, int64_t ldb, bm_stream_t stream);

/* Triangular band solve x <- op(A)^-1 x, BLAS xTBSV: uplo 'U'/'L', trans 'N'/'T'/'C',
 * diag 'N'/'U', any nonzero incx (negative: BLAS convention); A is the triangular band
 * (k+1) x n with lda >= k+1 (upper: diagonal in row k; lower: diagonal in row 0).  Each
 * element gets reference DTBSV's operations in its order (fused multiply-adds).
 * Replaces tbsv! (src/blas.jl:112-147) reached from UpperTriangular(A) \ b and
 * LowerTriangular(A) \ b (src/tribanded.jl:75-96), and banded QR's back-substitution. */
int bm_dtbsv(char uplo, char trans, char diag, int64_t n, int64_t k, const double *A, int64_t lda, double *x,
             int64_t incx, bm_stream_t stream);
int bm_stbsv(char uplo, char trans, char diag, int64_t n, int64_t k, const float *A, int64_t lda, float *x,
             int64_t incx, bm_stream_t stream);

/* Triangular band product x <- op(A) x, BLAS xTBMV, every uplo / trans / diag form,
 * any nonzero incx; storage as xTBSV.  Each output gets reference DTBMV's operations in
 * its order.  Replaces tbmv! (src/blas.jl:71-108) reached from UpperTriangular(A) * x
 * and LowerTriangular(A) * x (src/tribanded.jl:47-54). */
int bm_dtbmv(char uplo, char trans, char diag, int64_t n, int64_t k, const double *A, int64_t lda, double *x,
             int64_t incx, bm_stream_t stream);
int bm_stbmv(char uplo, char trans, char diag, int64_t n, int64_t k, const float *A, int64_t lda, float *x,
             int64_t incx, bm_stream_t stream);

/* Banded x dense: C <- alpha*A*B + beta*C for banded A (m x n, bandwidths (kl,ku),
 * lda >= kl+ku+1), dense B (n x k, ldb >= max(1,n)) and C (m x k, ldc >= max(1,m));
 * column c of C equals xGBMV 'N' of A with column c of B, bit for bit (the column loop
 * of materialize!(::MatMulMatAdd{<:BandedColumns,<:AbstractStridedLayout}),
 * src/generic/matmul.jl:243-256).  beta == 0: C is not read. */
int bm_dgbmm_bd(int64_t m, int64_t n, int64_t kl, int64_t ku, int64_t k, double alpha, const double *A, int64_t lda,
                const double *B, int64_t ldb, double beta, double *C, int64_t ldc, bm_stream_t stream);
int bm_sgbmm_bd(int64_t m, int64_t n, int64_t kl, int64_t ku, int64_t k, float alpha, const float *A, int64_t lda,
                const float *B, int64_t ldb, float beta, float *C, int64_t ldc, bm_stream_t stream);

/* Dense x banded: C <- alpha*D*A + beta*C for dense D (k x m, ldd >= max(1,k)),
 * banded A (m x n, (kl,ku), lda) and C (k x n, ldc >= max(1,k)); row r of C equals
 * xGBMV 'T' of A with row r of D, bit for bit (the row loop of
 * materialize!(::MatMulMatAdd{<:AbstractStridedLayout,<:BandedColumns}),
 * src/generic/matmul.jl:258-271). */
int bm_dgbmm_db(int64_t m, int64_t n, int64_t kl, int64_t ku, int64_t k, double alpha, const double *D, int64_t ldd,
                const double *A, int64_t lda, double beta, double *C, int64_t ldc, bm_stream_t stream);
int bm_sgbmm_db(int64_t m, int64_t n, int64_t kl, int64_t ku, int64_t k, float alpha, const float *D, int64_t ldd,
                const float *A, int64_t lda, float beta, float *C, int64_t ldc, bm_stream_t stream);

/* ------------------------------------------------------------------ symmetric band
 * Cholesky factorization of a symmetric positive definite band, LAPACK xPBTRF: AB is
 * the (kd+1) x n symmetric band storage (uplo 'U': A(i,j) at row kd+i-j for i <= j;
 * 'L': at row i-j for i >= j), ldab >= kd+1, overwritten by the factor U (A = U^T U) or
 * L (A = L L^T); *info (device) receives 0, or j > 0 when the leading minor of order j
 * is not positive definite (the factorization stops there).  Element for element the
 * unblocked xPBTF2 (bit for bit with it); kd <= 167 in Float64, 237 in Float32.
 * Replaces pbtrf! (src/lapack.jl:268-298) reached from banded_chol!
 * (src/symbanded/BandedCholesky.jl:2-12). */
int bm_dpbtrf(char uplo, int64_t n, int64_t kd, double *AB, int64_t ldab, int64_t *info, bm_stream_t stream);
int bm_spbtrf(char uplo, int64_t n, int64_t kd, float *AB, int64_t ldab, int64_t *info, bm_stream_t stream);

/* Solve A X = B with the xPBTRF factor (LAPACK xPBTRS: two triangular band sweeps per
 * right-hand side); B is n x nrhs, ldb >= max(1,n), overwritten with X.  Replaces
 * pbtrs! (src/lapack.jl:300-332). */
int bm_dpbtrs(char uplo, int64_t n, int64_t kd, int64_t nrhs, const double *AB, int64_t ldab, double *B, int64_t ldb,
              bm_stream_t stream);
int bm_spbtrs(char uplo, int64_t n, int64_t kd, int64_t nrhs, const float *AB, int64_t ldab, float *B, int64_t ldb,
              bm_stream_t stream);

/* y <- alpha*A*x + beta*y for a symmetric band A (k off-diagonals, storage as xPBTRF's),
 * BLAS xSBMV, any nonzero incx/incy; each output in reference DSBMV's order.  Replaces
 * sbmv! (src/blas.jl:35-64). */
int bm_dsbmv(char uplo, int64_t n, int64_t k, double alpha, const double *A, int64_t lda, const double *x,
             int64_t incx, double beta, double *y, int64_t incy, bm_stream_t stream);
int bm_ssbmv(char uplo, int64_t n, int64_t k, float alpha, const float *A, int64_t lda, const float *x, int64_t incx,
             float beta, float *y, int64_t incy, bm_stream_t stream);

/* ------------------------------------------------------------------ elementwise
 * Y <- a*X + Y for banded X (m x n, bandwidths (Xl,Xu), ldx) and Y ((Yl,Yu), ldy).
 * Equal bandwidths: BLAS axpy over the whole storage, y = fma(a, x, y) (axpy!(a, X.data,
 * Y.data), src/banded/BandedMatrix.jl:1006-1015).  Otherwise banded_generic_axpy!
 * (src/generic/broadcast.jl:978-1020): *bad (device) receives j*m + k of the first
 * (column-order) nonzero in-matrix entry X(k,j) outside Y's bands, in which case Y is
 * left untouched (the reference throws BandError); else *bad = UINT64_MAX and the
 * overlapping bands get y = a*x + y rounded twice (Julia does not fuse it). */
int bm_dgbaxpy(int64_t m, int64_t n, double a, int64_t Xl, int64_t Xu, const double *X, int64_t ldx, int64_t Yl,
               int64_t Yu, double *Y, int64_t ldy, unsigned long long *bad, bm_stream_t stream);
int bm_sgbaxpy(int64_t m, int64_t n, float a, int64_t Xl, int64_t Xu, const float *X, int64_t ldx, int64_t Yl,
               int64_t Yu, float *Y, int64_t ldy, unsigned long long *bad, bm_stream_t stream);

/* A <- alpha*A over the band storage (banded_lmul!, src/generic/broadcast.jl:960-965). */
int bm_dgbscal(int64_t m, int64_t n, int64_t l, int64_t u, double alpha, double *A, int64_t lda, bm_stream_t stream);
int bm_sgbscal(int64_t m, int64_t n, int64_t l, int64_t u, float alpha, float *A, int64_t lda, bm_stream_t stream);

/* A <- A + sigma*I: sigma added to the min(m,n) diagonal entries (storage row u; needs
 * l, u >= 0); the broadcast A + sigma*I of src/generic/broadcast.jl in place. */
int bm_dgbshift(int64_t m, int64_t n, int64_t l, int64_t u, double sigma, double *A, int64_t lda, bm_stream_t stream);
int bm_sgbshift(int64_t m, int64_t n, int64_t l, int64_t u, float sigma, float *A, int64_t lda, bm_stream_t stream);

/* *result (device) <- dot(x, A, y) = sum_j y_j sum_i A(i,j) x_i for banded A (m x n,
 * l, u >= 0), x of length m, y of length n; columns with y_j == 0 are skipped as in
 * _dot (src/banded/dot.jl:1-22).  work: 1024 device elements of scratch.  The column
 * sums run in ascending i with fused multiply-adds and the total is a fixed two-level
 * tree: deterministic, equal to the reference's @simd sum to rounding. */
int bm_dgbdot(int64_t m, int64_t n, int64_t l, int64_t u, const double *x, const double *A, int64_t lda,
              const double *y, double *result, double *work, bm_stream_t stream);
int bm_sgbdot(int64_t m, int64_t n, int64_t l, int64_t u, const float *x, const float *A, int64_t lda, const float *y,
              float *result, float *work, bm_stream_t stream);

/* ------------------------------------------------------------------ conversion
 * sparse(A) for an m x n band (l, u) as CSC arrays on the device: colptr (n+1 int64,
 * 0-based), rowval and nzval (bm_gb2csc_nnz(m, n, l, u) entries).  Every in-matrix band
 * slot is a stored entry (zeros included); a column without one keeps one structural
 * zero at the clamped row, as sparse(_banded_rowval, _banded_colval, _banded_nzval)
 * builds it (ext/BandedMatricesSparseArraysExt.jl:7-9, src/banded/BandedMatrix.jl:
 * 796-836). */
int64_t bm_gb2csc_nnz(int64_t m, int64_t n, int64_t l, int64_t u);
int bm_dgb2csc(int64_t m, int64_t n, int64_t l, int64_t u, const double *A, int64_t lda, int64_t *colptr,
               int64_t *rowval, double *nzval, bm_stream_t stream);
int bm_sgb2csc(int64_t m, int64_t n, int64_t l, int64_t u, const float *A, int64_t lda, int64_t *colptr,
               int64_t *rowval, float *nzval, bm_stream_t stream);

/* lu[0], lu[1] (device) <- bandwidths(S) of a CSC matrix (m x n; colptr/rowval 0-based):
 * the extreme diagonals of its nonzero values, -max(m,n) each when every stored value is
 * zero, -40320 each (bandwidths(Zeros)) when nothing is stored (the extension's
 * bandwidths(::SparseMatrixCSC), ext/BandedMatricesSparseArraysExt.jl:11-33). */
int bm_dcsc_bandwidths(int64_t m, int64_t n, const int64_t *colptr, const int64_t *rowval, const double *nzval,
                       int64_t *lu, bm_stream_t stream);
int bm_scsc_bandwidths(int64_t m, int64_t n, const int64_t *colptr, const int64_t *rowval, const float *nzval,
                       int64_t *lu, bm_stream_t stream);

/* BandedMatrix(S, (l, u)): the band storage A ((l+u+1) x n, lda) zeroed and filled from
 * the CSC matrix S; *dropped (device) counts nonzero entries outside the band (not
 * stored). */
int bm_dcsc2gb(int64_t m, int64_t n, const int64_t *colptr, const int64_t *rowval, const double *nzval, int64_t l,
               int64_t u, double *A, int64_t lda, unsigned long long *dropped, bm_stream_t stream);
int bm_scsc2gb(int64_t m, int64_t n, const int64_t *colptr, const int64_t *rowval, const float *nzval, int64_t l,
               int64_t u, float *A, int64_t lda, unsigned long long *dropped, bm_stream_t stream);

/* Row-major band data to column-major band storage (the BandedRows copy of
 * _BandedMatrix(::BandedRows, A), src/banded/BandedMatrix.jl:267-284): R is m x (l+u+1)
 * column-major (ldr >= m) with A(i, c) at R[i + (c - i + l) * ldr]; the in-matrix slots
 * of A ((l+u+1) x n, lda) are written. */
int bm_dgbrows2cols(int64_t m, int64_t n, int64_t l, int64_t u, const double *R, int64_t ldr, double *A, int64_t lda,
                    bm_stream_t stream);
int bm_sgbrows2cols(int64_t m, int64_t n, int64_t l, int64_t u, const float *R, int64_t ldr, float *A, int64_t lda,
                    bm_stream_t stream);

/* ------------------------------------------------------------------ adjoint
 * Reverse-mode derivative of X = A \ B for an upstream gradient W = dL/dX (all
 * n x nrhs, leading dim n), with A's xGBTRF factors (LU, ldab, ipiv):
 *   grad_B    <- A^{-T} W                      (transposed xGBTRS on the factors)
 *   grad_band <- -(A^{-T} W) X^T on A's band   (BLAS band layout, (kl+ku+1) x n,
 *                                               leading dim ldg; NULL to skip)
 * X may be NULL: it is then recomputed from B into Xwork (n x nrhs workspace).  LU,
 * ipiv, W and grad_B are read or written only when n > 0 and nrhs > 0, and must then
 * be non-NULL (-5, -7, -10, -11).  No counterpart in the reference; it is the rrule of \ built on the transposed solve
 * ldiv!(transpose(F), B) (src/banded/linalg.jl:41-47). */
int bm_dgbsv_adjoint(int64_t n, int64_t kl, int64_t ku, int64_t nrhs, const double *LU, int64_t ldab,
                     const int64_t *ipiv, const double *X, const double *B, const double *W, double *grad_B,
                     double *grad_band, int64_t ldg, double *Xwork, bm_stream_t stream);
int bm_sgbsv_adjoint(int64_t n, int64_t kl, int64_t ku, int64_t nrhs, const float *LU, int64_t ldab,
                     const int64_t *ipiv, const float *X, const float *B, const float *W, float *grad_B,
                     float *grad_band, int64_t ldg, float *Xwork, bm_stream_t stream);

/* ------------------------------------------------------------------ batched
 * One square system of a batch: its band (gbtrf storage) at AB + ab_offset, its
 * right-hand sides at B + b_offset (n x nrhs, leading dim ldb), its pivots at
 * ipiv + ipiv_offset.  Systems may differ in n, kl, ku and nrhs. */
typedef struct {
  int64_t n, kl, ku, nrhs;
  int64_t ab_offset, ldab;
  int64_t b_offset, ldb;
  int64_t ipiv_offset;
} bm_gb_desc;

/* Factor and solve every system of a batch in one persistent launch: warps take
 * systems from a device work queue in the order `order` (device int32 list of
 * system indices, most expensive first; NULL = natural order).  info[s] (device)
 * receives system s's gbtrf info; systems with info != 0 are not solved.  The
 * kernel checks every descriptor before it touches the system: an illegal field, or
 * a kl/ku above the bounds shared memory was sized for (max_kl/max_ku, or the
 * schedule's), gives info[s] = -(field number: n 1, kl 2, ku 3, nrhs 4, ab_offset 5,
 * ldab 6, b_offset 7, ldb 8, ipiv_offset 9) and the system is skipped; order entries
 * outside [0, count) are skipped.
 * `counter` is one device int32 of workspace (reset by the call).  max_kl/max_ku
 * bound the bandwidths in the batch (shared memory is sized from them).  No
 * allocation, no host synchronisation: the call can be captured in a CUDA graph.
 * No counterpart in the reference (which solves one system per call); per
 * system it equals lu! + ldiv! (src/banded/BandedLU.jl:90-103, linalg.jl:24-30). */
int bm_dgbsv_batched(int64_t count, const bm_gb_desc *descs, const int32_t *order, double *AB, int64_t *ipiv,
                     double *B, int64_t *info, int32_t *counter, int64_t max_kl, int64_t max_ku, bm_stream_t stream);
int bm_sgbsv_batched(int64_t count, const bm_gb_desc *descs, const int32_t *order, float *AB, int64_t *ipiv,
                     float *B, int64_t *info, int32_t *counter, int64_t max_kl, int64_t max_ku, bm_stream_t stream);

/* Launch schedule of a batched solve.  order[0..n_wide) ("wide" systems) are solved
 * one at a time by a CTA of `warps` (4 or 8) warps; order[n_wide..count) ("narrow")
 * one per warp, each warp taking the next narrow system as it finishes.  wide_kl/ku
 * and narrow_kl/ku bound the bandwidths of each part (shared memory is sized from
 * them).  The host mirror's autotuner (BandedBatch.tune) times candidate schedules
 * on the batch itself and keeps the fastest. */
typedef struct {
  int64_t n_wide;
  int64_t warps;
  int64_t wide_kl, wide_ku;
  int64_t narrow_kl, narrow_ku;
} bm_gb_schedule;

/* bm_{d,s}gbsv_batched with an explicit schedule (sched: host pointer, read during
 * the call; order must list the wide systems first).  Graph-capturable like the
 * single-part entry points. */
int bm_dgbsv_batched_sched(int64_t count, const bm_gb_desc *descs, const int32_t *order, const bm_gb_schedule *sched,
                           double *AB, int64_t *ipiv, double *B, int64_t *info, int32_t *counter, bm_stream_t stream);
int bm_sgbsv_batched_sched(int64_t count, const bm_gb_desc *descs, const int32_t *order, const bm_gb_schedule *sched,
                           float *AB, int64_t *ipiv, float *B, int64_t *info, int32_t *counter, bm_stream_t stream);

/* Mixed-precision refined batched solve (LAPACK DSGESV's scheme on band storage):
 * each system's FP64 band (AB, gbtrf storage, matrix in rows kl..; read only) is
 * rounded to FP32 into AB32 (same offsets) and factored in FP32 with partial
 * pivoting; every right-hand side B (read only) is solved in FP32 and refined with
 * FP64 residuals r = b - A x and FP64 updates until the backward error
 * ||r||_inf / (||A||_inf ||x||_inf + ||b||_inf) <= tol or maxit corrections.  X
 * receives the solutions (B's layout), iters/berr the corrections taken and the
 * final backward error per system (max over its right-hand sides), info the FP32
 * factorization's info (or -(field number) for a descriptor the kernel rejects, as
 * in bm_dgbsv_batched; such a system is neither factored nor refined).  R32 is FP32
 * workspace laid out like B but with leading
 * dimension n (n*nrhs floats per system at its b_offset); counter is 4 int32 of
 * workspace.  kl + ku <= 256 per system; maxit is capped at 100.  The call enqueues
 * a factor launch, then maxit pairs of correction / FP64-residual launches (pairs
 * after every system has converged return at once).  No counterpart in the
 * reference; per system it replaces lu! + ldiv! (src/banded/BandedLU.jl:90-103,
 * src/banded/linalg.jl:24-30) when the caller accepts a backward-error target. */
int bm_dsgbsv_batched(int64_t count, const bm_gb_desc *descs, const int32_t *order, const double *AB,
                      const double *B, double *X, int64_t *ipiv, int64_t *info, float *AB32, float *R32,
                      int32_t *iters, double *berr, int32_t *counter, double tol, int64_t maxit, int64_t max_kl,
                      int64_t max_ku, bm_stream_t stream);

/* bm_dsgbsv_batched with an explicit schedule (see bm_gb_schedule). */
int bm_dsgbsv_batched_sched(int64_t count, const bm_gb_desc *descs, const int32_t *order, const bm_gb_schedule *sched,
                            const double *AB, const double *B, double *X, int64_t *ipiv, int64_t *info, float *AB32,
                            float *R32, int32_t *iters, double *berr, int32_t *counter, double tol, int64_t maxit,
                            bm_stream_t stream);

/* Mixed-precision refined solve of ONE banded system (LAPACK DSGESV's scheme on band
 * storage): the FP64 band AB ((kl+ku+1) x n, ldab >= kl+ku+1, A(i,c) at row ku+i-c, as
 * BandedMatrix stores it; read only) is factored in FP32 with partial pivoting -- for
 * 64 <= kl+ku <= 256 and kl <= 224 by the tensor-core blocked LU (trailing updates as
 * kind::tf32 MMAs with hi/lo-split operands, FP32-level products), otherwise by the
 * FP32 form of bm_sgbtrf -- and every right-hand side B (n x nrhs, ldb) is solved in
 * FP32 and refined with FP64 residuals r = b - A x and FP64 updates until the
 * backward error max_c ||r_c||_inf / (||A||_inf ||x_c||_inf + ||b_c||_inf) <= tol or
 * maxit corrections (capped at 100).  X (n x nrhs, ldx) receives the solutions, ipiv
 * the FP32 factorization's pivots, *info (device) its info (> 0: exactly singular in
 * FP32; nothing is solved and *berr is +inf), *iter (device int32) the corrections
 * taken, *berr (device double) the final backward error.  Workspace: swork, FP32,
 * 16-byte aligned, ldf*n + n*nrhs floats with ldf = 2kl+ku+1 rounded up to a multiple
 * of 4 (the factors in gbtrf layout with leading dimension ldf, then the correction);
 * work, FP64, n*nrhs + 3*nrhs + 2 doubles.  kl + ku <= 256.  The whole loop is
 * enqueued at once and decided on the device (a flag turns the remaining launches
 * into no-ops): no host synchronisation, no allocation.  No counterpart in the
 * reference; it replaces lu! + ldiv! (src/banded/BandedLU.jl:90-103,
 * src/banded/linalg.jl:24-30) for a caller that accepts a backward-error target. */
int bm_dsgbsv(int64_t n, int64_t kl, int64_t ku, int64_t nrhs, const double *AB, int64_t ldab, const double *B,
              int64_t ldb, double *X, int64_t ldx, int64_t *ipiv, float *swork, double *work, double tol,
              int64_t maxit, int32_t *iter, double *berr, int64_t *info, bm_stream_t stream);

/* The tensor-core FP32 factorization of bm_dsgbsv alone: AB as there, F the FP32 gbtrf
 * storage ((2kl+ku+1) x n, ldf >= 2kl+ku+1) receiving L and U in the layout xGBTRS
 * reads, ipiv n 1-based pivots, *info (device) LAPACK's info.  Needs 64 <= kl+ku <= 256
 * and kl <= 224 (else BM_ERR_UNSUPPORTED).  The pivot is the largest |a| to 2^-15
 * relative (the first row among near-equal magnitudes).  No counterpart in the
 * reference (dgbtrf of lu!, src/banded/BandedLU.jl:98, in FP32 on tensor cores). */
int bm_sgbtrf_tc(int64_t n, int64_t kl, int64_t ku, const double *AB, int64_t ldab, float *F, int64_t ldf,
                 int64_t *ipiv, int64_t *info, bm_stream_t stream);

/* Plans: the autotuned schedule of a batch and its device workspace, owned by the
 * library.  bm_plan_create times every candidate bm_gb_schedule (4 or 8 warps per CTA x
 * the wide/narrow split at 0, 8, 16, 24, 32, 48, 64, 96 or all band columns) on a copy
 * of the batch (AB, B: device buffers laid out by the descriptors; not modified) for the
 * plain FP64 solve (kind 0) or the refined solve (kind 1), keeps the fastest, and
 * stores its processing order and work counters in device memory it allocates; the
 * choice is cached per (device, batch shape) for the process.  host_descs is a host copy
 * of the count descriptors in descs (device).  It allocates and synchronises: call it
 * once, outside any stream capture.  The executions enqueue the scheduled solve with
 * no allocation and no synchronisation.  No counterpart in the reference (which
 * solves one system per call). */
typedef struct bm_plan_st *bm_plan;
int bm_plan_create(bm_plan *plan, int64_t count, const bm_gb_desc *host_descs, const bm_gb_desc *descs, int kind,
                   const double *AB, const double *B, bm_stream_t stream);
int bm_plan_destroy(bm_plan plan);
/* The plan's schedule, the time of its timing run (ms) and the candidates timed. */
int bm_plan_schedule(bm_plan plan, bm_gb_schedule *sched, double *tuned_ms, int64_t *candidates);
/* bm_dgbsv_batched_sched with the plan's schedule (kind 0). */
int bm_plan_execute_dgbsv(bm_plan plan, const bm_gb_desc *descs, double *AB, int64_t *ipiv, double *B, int64_t *info,
                          bm_stream_t stream);
/* bm_dsgbsv_batched_sched with the plan's schedule (kind 1). */
int bm_plan_execute_dsgbsv(bm_plan plan, const bm_gb_desc *descs, const double *AB, const double *B, double *X,
                           int64_t *ipiv, int64_t *info, float *AB32, float *R32, int32_t *iters, double *berr,
                           double tol, int64_t maxit, bm_stream_t stream);

/* Allocation-free variant of bm_dgbsv_batched, for callers that cannot allocate
 * device memory when they solve: real-time loops that must not block on an
 * allocator, and hosts whose device memory belongs to another runtime's pool (Julia's
 * CUDA.jl, PyTorch) and that cannot hand the library a workspace.  The caller passes
 * only inputs and outputs; the work queue and the longest-first order live in a
 * 256 KiB static device array inside the library, which every GPU that loads the
 * library keeps until exit.  At most 65536 systems per call (more:
 * BM_ERR_UNSUPPORTED, see bm_last_error()).  The first call on a device looks up the
 * array's address (once per device, cached for the process; after cudaDeviceReset
 * reload the library) and should come before any stream capture.  All calls share
 * the array, so calls that overlap on the GPU (concurrent streams) race; serialise
 * them.  No counterpart in the reference. */
int bm_dgbsv_batched_noalloc(int64_t count, const bm_gb_desc *descs, double *AB, int64_t *ipiv, double *B,
                             int64_t *info, int64_t max_kl, int64_t max_ku, bm_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* BANDEDGPU_H */
