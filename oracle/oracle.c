/*
 * CPU oracle for the banded hot path.  TEST INFRASTRUCTURE ONLY: it is the
 * checker that the CUDA library is compared against, never part of the
 * product path.  Only tests/, __graft_entry__.smoke() and the CPU-baseline
 * leg of bench.py load it.
 *
 * BandedMatrices.jl does the arithmetic of this path in two places:
 *   - third-party BLAS/LAPACK (OpenBLAS through libblastrampoline), reached by
 *     ccall: dgbmv_ (src/blas.jl:19-26, stdlib BLAS.gbmv! from
 *     src/generic/matmul.jl:22), dgbtrf_ (LAPACK.gbtrf! from
 *     src/banded/BandedLU.jl:98), dgbtrs_ (src/banded/linalg.jl:28,46),
 *     dtbsv_ (src/blas.jl:134 via src/tribanded.jl:82).  These are the
 *     reference LAPACK 3.x algorithms dgbtf2/dgbtrs and reference BLAS
 *     dgbmv/dger/dgemv/dtbsv, restated here in C (0-based).  OpenBLAS is not
 *     pinned by the reference (no Manifest; Project.toml:34 only says
 *     julia = "1.10").  The restatement is pinned against the OpenBLAS build
 *     that SciPy bundles (tests/test_oracle.py, tests/golden/).
 *   - pure Julia: _gbmm! (src/banded/gbmm.jl:296-340, column kernels :18-158),
 *     banded_mul! (src/generic/matmul.jl:143-172), _banded_qr!
 *     (src/banded/bandedqr.jl:13-28) with reflector!/reflectorApply! from
 *     LinearAlgebra/ArrayLayouts, banded_qr_lmul! (bandedqr.jl:38-94).
 *
 * Floating-point contract: compiled with -ffp-contract=off; every
 * multiply-add that a BLAS kernel performs as an update (dger, dgbmv 'N',
 * the dtbsv sweeps) is written as an explicit fma() so that the result is
 * identical on x86-64 and aarch64 hosts and bit-comparable with the CUDA
 * kernels, which use the same fused updates in the same order.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

typedef int64_t i64;

static inline i64 imin(i64 a, i64 b) { return a < b ? a : b; }
static inline i64 imax(i64 a, i64 b) { return a > b ? a : b; }

#define DEFINE_ALL(T, P, FMA, ABS, SQRT, COPYSIGN)                                              \
                                                                                                \
/* y := alpha*op(A)*x + beta*y, A in BLAS band storage (kl+ku+1 rows, leading dim lda).       */ \
/* Reference BLAS xGBMV loop order; 'N' is column-oriented (axpy), 'T' is dot-oriented.        */ \
int P##gbmv(char trans, i64 m, i64 n, i64 kl, i64 ku, T alpha, const T *a, i64 lda,           \
            const T *x, i64 incx, T beta, T *y, i64 incy)                                       \
{                                                                                               \
    int notr = (trans == 'N' || trans == 'n');                                                  \
    if (!notr && !(trans == 'T' || trans == 't' || trans == 'C' || trans == 'c')) return -1;    \
    if (m < 0) return -2;                                                                       \
    if (n < 0) return -3;                                                                       \
    if (kl < 0) return -4;                                                                      \
    if (ku < 0) return -5;                                                                      \
    if (lda < kl + ku + 1) return -8;                                                           \
    if (incx == 0) return -10;                                                                  \
    if (incy == 0) return -13;                                                                  \
    if (m == 0 || n == 0 || (alpha == 0 && beta == 1)) return 0;                                \
    i64 lenx = notr ? n : m, leny = notr ? m : n;                                               \
    i64 kx = incx > 0 ? 0 : -(lenx - 1) * incx;                                                 \
    i64 ky = incy > 0 ? 0 : -(leny - 1) * incy;                                                 \
    if (beta != 1) {                                                                            \
        for (i64 i = 0, iy = ky; i < leny; i++, iy += incy)                                     \
            y[iy] = (beta == 0) ? (T)0 : beta * y[iy];                                          \
    }                                                                                           \
    if (alpha == 0) return 0;                                                                   \
    if (notr) {                                                                                 \
        for (i64 j = 0, jx = kx; j < n; j++, jx += incx) {                                      \
            T temp = alpha * x[jx];                                                             \
            i64 k = ku - j;                                                                     \
            i64 i0 = imax(0, j - ku), i1 = imin(m - 1, j + kl);                                 \
            for (i64 i = i0; i <= i1; i++)                                                      \
                y[ky + i * incy] = FMA(temp, a[(k + i) + j * lda], y[ky + i * incy]);           \
        }                                                                                       \
    } else {                                                                                    \
        for (i64 j = 0, jy = ky; j < n; j++, jy += incy) {                                      \
            T temp = 0;                                                                         \
            i64 k = ku - j;                                                                     \
            i64 i0 = imax(0, j - ku), i1 = imin(m - 1, j + kl);                                 \
            for (i64 i = i0; i <= i1; i++)                                                      \
                temp = FMA(a[(k + i) + j * lda], x[kx + i * incx], temp);                       \
            y[jy] = FMA(alpha, temp, y[jy]);                                                    \
        }                                                                                       \
    }                                                                                           \
    return 0;                                                                                   \
}                                                                                               \
                                                                                                \
/* Unblocked LAPACK xGBTF2: partial-pivot LU in gbtrf storage (ldab >= 2kl+ku+1),             */ \
/* A(i,c) = ab[(kl+ku+i-c) + c*ldab].  ipiv is written 1-based (Julia/LAPACK convention).     */ \
int P##gbtf2(i64 m, i64 n, i64 kl, i64 ku, T *ab, i64 ldab, i64 *ipiv, i64 *info)             \
{                                                                                               \
    *info = 0;                                                                                  \
    if (m < 0) return -1;                                                                       \
    if (n < 0) return -2;                                                                       \
    if (kl < 0) return -3;                                                                      \
    if (ku < 0) return -4;                                                                      \
    if (ldab < 2 * kl + ku + 1) return -6;                                                      \
    if (m == 0 || n == 0) return 0;                                                             \
    const i64 kv = ku + kl;                                                                     \
    /* zero the fill-in above the U band in columns ku+1 .. min(kv,n)-1 */                      \
    for (i64 j = ku + 1; j < imin(kv, n); j++)                                                  \
        for (i64 r = kv - j; r < kl; r++) ab[r + j * ldab] = 0;                                 \
    i64 ju = 0;                                                                                 \
    for (i64 j = 0; j < imin(m, n); j++) {                                                      \
        if (j + kv < n)                                                                         \
            for (i64 r = 0; r < kl; r++) ab[r + (j + kv) * ldab] = 0;                           \
        i64 km = imin(kl, m - 1 - j);                                                           \
        T *col = ab + kv + j * ldab; /* col[i] = A(j+i, j) */                                   \
        i64 jp = 0;                                                                             \
        T amax = ABS(col[0]);                                                                   \
        for (i64 i = 1; i <= km; i++)                                                           \
            if (ABS(col[i]) > amax) { amax = ABS(col[i]); jp = i; }                             \
        ipiv[j] = j + jp + 1;                                                                   \
        if (col[jp] != 0) {                                                                     \
            ju = imax(ju, imin(j + ku + jp, n - 1));                                            \
            if (jp != 0) {                                                                      \
                for (i64 c = j; c <= ju; c++) {                                                 \
                    T *p1 = ab + (kv + j - c) + c * ldab;                                       \
                    T *p2 = ab + (kv + j + jp - c) + c * ldab;                                  \
                    T t = *p1; *p1 = *p2; *p2 = t;                                              \
                }                                                                               \
            }                                                                                   \
            if (km > 0) {                                                                       \
                T r = (T)1 / col[0];                                                            \
                for (i64 i = 1; i <= km; i++) col[i] = r * col[i];                              \
                for (i64 c = j + 1; c <= ju; c++) {                                             \
                    T uc = ab[(kv + j - c) + c * ldab];                                         \
                    if (uc != 0) {                                                              \
                        T temp = -uc;                                                           \
                        for (i64 i = 1; i <= km; i++) {                                         \
                            T *p = ab + (kv + j + i - c) + c * ldab;                            \
                            *p = FMA(col[i], temp, *p);                                         \
                        }                                                                       \
                    }                                                                           \
                }                                                                               \
            }                                                                                   \
        } else if (*info == 0) {                                                                \
            *info = j + 1;                                                                      \
        }                                                                                       \
    }                                                                                           \
    return 0;                                                                                   \
}                                                                                               \
                                                                                                \
/* Reference BLAS xTBSV, upper/lower, 'N'/'T', unit/non-unit, incx=1 only.                     */ \
int P##tbsv(char uplo, char trans, char diag, i64 n, i64 k, const T *a, i64 lda, T *x)          \
{                                                                                               \
    int upper = (uplo == 'U' || uplo == 'u');                                                   \
    int notr = (trans == 'N' || trans == 'n');                                                  \
    int nounit = (diag == 'N' || diag == 'n');                                                  \
    if (n < 0) return -4;                                                                       \
    if (k < 0) return -5;                                                                       \
    if (lda < k + 1) return -7;                                                                 \
    if (n == 0) return 0;                                                                       \
    if (notr) {                                                                                 \
        if (upper) {                                                                            \
            for (i64 j = n - 1; j >= 0; j--) {                                                  \
                if (x[j] != 0) {                                                                \
                    i64 l = k - j;                                                              \
                    if (nounit) x[j] = x[j] / a[k + j * lda];                                   \
                    T temp = -x[j];                                                             \
                    for (i64 i = j - 1; i >= imax(0, j - k); i--)                               \
                        x[i] = FMA(temp, a[(l + i) + j * lda], x[i]);                           \
                }                                                                               \
            }                                                                                   \
        } else {                                                                                \
            for (i64 j = 0; j < n; j++) {                                                       \
                if (x[j] != 0) {                                                                \
                    i64 l = -j;                                                                 \
                    if (nounit) x[j] = x[j] / a[0 + j * lda];                                   \
                    T temp = -x[j];                                                             \
                    for (i64 i = j + 1; i <= imin(n - 1, j + k); i++)                           \
                        x[i] = FMA(temp, a[(l + i) + j * lda], x[i]);                           \
                }                                                                               \
            }                                                                                   \
        }                                                                                       \
    } else {                                                                                    \
        if (upper) {                                                                            \
            for (i64 j = 0; j < n; j++) {                                                       \
                T temp = x[j];                                                                  \
                i64 l = k - j;                                                                  \
                for (i64 i = imax(0, j - k); i < j; i++)                                        \
                    temp = FMA(-a[(l + i) + j * lda], x[i], temp);                              \
                if (nounit) temp = temp / a[k + j * lda];                                       \
                x[j] = temp;                                                                    \
            }                                                                                   \
        } else {                                                                                \
            for (i64 j = n - 1; j >= 0; j--) {                                                  \
                T temp = x[j];                                                                  \
                i64 l = -j;                                                                     \
                for (i64 i = imin(n - 1, j + k); i > j; i--)                                    \
                    temp = FMA(-a[(l + i) + j * lda], x[i], temp);                              \
                if (nounit) temp = temp / a[0 + j * lda];                                       \
                x[j] = temp;                                                                    \
            }                                                                                   \
        }                                                                                       \
    }                                                                                           \
    return 0;                                                                                   \
}                                                                                               \
                                                                                                \
/* LAPACK xGBTRS: solve op(A) X = B with the xGBTRF factors.  ipiv is 1-based.                */ \
int P##gbtrs(char trans, i64 n, i64 kl, i64 ku, i64 nrhs, const T *ab, i64 ldab,              \
             const i64 *ipiv, T *b, i64 ldb)                                                    \
{                                                                                               \
    int notr = (trans == 'N' || trans == 'n');                                                  \
    if (!notr && !(trans == 'T' || trans == 't' || trans == 'C' || trans == 'c')) return -1;    \
    if (n < 0) return -2;                                                                       \
    if (kl < 0) return -3;                                                                      \
    if (ku < 0) return -4;                                                                      \
    if (nrhs < 0) return -5;                                                                    \
    if (ldab < 2 * kl + ku + 1) return -7;                                                      \
    if (ldb < imax(1, n)) return -10;                                                           \
    if (n == 0 || nrhs == 0) return 0;                                                          \
    const i64 kv = kl + ku;                                                                     \
    if (notr) {                                                                                 \
        if (kl > 0) {                                                                           \
            for (i64 j = 0; j < n - 1; j++) {                                                   \
                i64 lm = imin(kl, n - 1 - j);                                                   \
                i64 l = ipiv[j] - 1;                                                            \
                if (l != j)                                                                     \
                    for (i64 r = 0; r < nrhs; r++) {                                            \
                        T t = b[l + r * ldb]; b[l + r * ldb] = b[j + r * ldb]; b[j + r * ldb] = t; \
                    }                                                                           \
                const T *lc = ab + kv + 1 + j * ldab;                                           \
                for (i64 r = 0; r < nrhs; r++) {                                                \
                    T bj = b[j + r * ldb];                                                      \
                    if (bj != 0) {                                                              \
                        T temp = -bj;                                                           \
                        for (i64 i = 0; i < lm; i++)                                            \
                            b[j + 1 + i + r * ldb] = FMA(lc[i], temp, b[j + 1 + i + r * ldb]);  \
                    }                                                                           \
                }                                                                               \
            }                                                                                   \
        }                                                                                       \
        for (i64 r = 0; r < nrhs; r++) P##tbsv('U', 'N', 'N', n, kv, ab, ldab, b + r * ldb);    \
    } else {                                                                                    \
        for (i64 r = 0; r < nrhs; r++) P##tbsv('U', 'T', 'N', n, kv, ab, ldab, b + r * ldb);    \
        if (kl > 0) {                                                                           \
            for (i64 j = n - 2; j >= 0; j--) {                                                  \
                i64 lm = imin(kl, n - 1 - j);                                                   \
                const T *lc = ab + kv + 1 + j * ldab;                                           \
                for (i64 r = 0; r < nrhs; r++) {                                                \
                    T temp = 0;                                                                 \
                    for (i64 i = 0; i < lm; i++)                                                \
                        temp = FMA(b[j + 1 + i + r * ldb], lc[i], temp);                        \
                    b[j + r * ldb] = FMA((T)-1, temp, b[j + r * ldb]);                          \
                }                                                                               \
                i64 l = ipiv[j] - 1;                                                            \
                if (l != j)                                                                     \
                    for (i64 r = 0; r < nrhs; r++) {                                            \
                        T t = b[l + r * ldb]; b[l + r * ldb] = b[j + r * ldb]; b[j + r * ldb] = t; \
                    }                                                                           \
            }                                                                                   \
        }                                                                                       \
    }                                                                                           \
    return 0;                                                                                   \
}                                                                                               \
                                                                                                \
/* Generic banded product, the arithmetic of banded_mul! (src/generic/matmul.jl:143-172)      */ \
/* extended with alpha/beta: C = alpha*A*B + beta*C on C's in-product bands, C's extra bands  */ \
/* beta-scaled (zeroed when beta == 0, C not read), as gbmm! does (gbmm.jl:286-288).          */ \
/* A: n x nu (Al,Au), B: nu x m (Bl,Bu), C: n x m (Cl,Cu); all bandwidths >= 0 and            */ \
/* Cl >= Al+Bl, Cu >= Au+Bu (the case gbmm! handles without pruning).                          */ \
int P##gbmm_generic(i64 n, i64 nu, i64 m, i64 Al, i64 Au, i64 Bl, i64 Bu, i64 Cl, i64 Cu,       \
                    T alpha, const T *A, i64 lda, const T *B, i64 ldb, T beta, T *C, i64 ldc)   \
{                                                                                               \
    if (Al < 0 || Au < 0 || Bl < 0 || Bu < 0 || Cl < Al + Bl || Cu < Au + Bu) return -4;        \
    const i64 pl = Al + Bl, pu = Au + Bu;                                                       \
    for (i64 j = 0; j < m; j++) {                                                               \
        for (i64 k = imax(0, j - Cu); k <= imin(n - 1, j + Cl); k++) {                          \
            T *cp = C + (Cu + k - j) + j * ldc;                                                 \
            T cold = (beta == 0) ? (T)0 : beta * *cp;                                           \
            if (k < j - pu || k > j + pl) { *cp = cold; continue; }                             \
            i64 v0 = imax(imax(0, k - Al), j - Bu), v1 = imin(imin(nu - 1, k + Au), j + Bl);    \
            T tmp = 0;                                                                          \
            for (i64 v = v0; v <= v1; v++)                                                      \
                tmp = FMA(A[(Au + k - v) + v * lda], B[(Bu + v - j) + j * ldb], tmp);           \
            *cp = FMA(alpha, tmp, cold);                                                        \
        }                                                                                       \
    }                                                                                           \
    return 0;                                                                                   \
}                                                                                               \
                                                                                                \
/* _gbmm! (gbmm.jl:296-340): each column of C is one small xGBMV over a window of A,          */ \
/* through the three column kernels A11_Btop_Ctop (:18-45), Atop_Bmid_Ctop (:57-86),           */ \
/* Amid_Bmid_Cmid (:99-127) and the trailing beta-scaling (:339).  Here C has exactly          */ \
/* (Cl,Cu) = (Al+Bl, Au+Bu) bands (the view gbmm! passes after scaling extra bands).           */ \
int P##gbmm_percol(i64 n, i64 nu, i64 m, i64 Al, i64 Au, i64 Bl, i64 Bu,                        \
                   T alpha, const T *a, i64 sta, const T *b, i64 stb, T beta, T *c, i64 stc)    \
{                                                                                               \
    const i64 Cl = Al + Bl, Cu = Au + Bu;                                                       \
    if (n == 0 || m == 0) return 0;                                                             \
    /* Julia j is 1-based below, pointers are offset with the same formulas as gbmm.jl */       \
    for (i64 j = 1; j <= imin(m, 1 + Bu); j++)                                                  \
        P##gbmv('N', imin(Cl + j, n), imin(Bl + j, nu), Al, Au, alpha, a, sta,                  \
                b + ((j - 1) * stb + Bu - j + 1), 1, beta, c + ((j - 1) * stc + Cu - j + 1), 1); \
    for (i64 j = 2 + Bu; j <= imin(imin(1 + Cu, nu + Bu), m); j++)                              \
        P##gbmv('N', imin(Cl + j, n), imin(Bl + Bu + 1, nu - j + Bu + 1), Al + j - Bu - 1,     \
                Au - j + Bu + 1, alpha, a + (j - Bu - 1) * sta, sta, b + (j - 1) * stb, 1, beta, \
                c + ((j - 1) * stc + Cu - j + 1), 1);                                           \
    for (i64 j = 2 + Cu; j <= imin(imin(m, nu + Bu), n + Cu); j++)                              \
        P##gbmv('N', imin(Cl + Cu + 1, n - j + Cu + 1), imin(Bl + Bu + 1, nu - (j - Bu) + 1),  \
                Al + Au, 0, alpha, a + (j - Bu - 1) * sta, sta, b + (j - 1) * stb, 1, beta,     \
                c + (j - 1) * stc, 1);                                                          \
    for (i64 j = nu + Bu + 1; j <= imin(m, n + Cu); j++)                                        \
        for (i64 r = 0; r < Cl + Cu + 1; r++) {                                                 \
            T *p = c + (j - 1) * stc + r;                                                       \
            *p = (beta == 0) ? (T)0 : beta * *p;                                                \
        }                                                                                       \
    return 0;                                                                                   \
}                                                                                               \
                                                                                                \
/* Euclidean norm (BLAS xNRM2, which LinearAlgebra.norm calls for strided vectors).    */ \
/* Squares are summed in four interleaved partial sums (element i goes to sum i mod 4,  */ \
/* each accumulated with fma in ascending i), combined as (s0+s1)+(s2+s3), the order of */ \
/* a 4-lane SIMD kernel.  When max|x| is inside a safe range the squares are taken      */ \
/* directly; otherwise each element is first divided by max|x| (overflow-safe).         */ \
static T P##nrm2(const T *x, i64 n)                                                             \
{                                                                                               \
    T scale = 0;                                                                                \
    for (i64 i = 0; i < n; i++) if (ABS(x[i]) > scale) scale = ABS(x[i]);                       \
    if (scale == 0 || !isfinite(scale)) return scale;                                           \
    const int direct = (sizeof(T) == 8) ? (scale > 0x1p-400 && scale < 0x1p400)                 \
                                        : (scale > 0x1p-50f && scale < 0x1p50f);                \
    T s4[4] = {0, 0, 0, 0};                                                                     \
    for (i64 i = 0; i < n; i++) {                                                               \
        T t = direct ? x[i] : x[i] / scale;                                                     \
        s4[i & 3] = FMA(t, t, s4[i & 3]);                                                       \
    }                                                                                           \
    T ssq = (s4[0] + s4[1]) + (s4[2] + s4[3]);                                                  \
    return direct ? SQRT(ssq) : scale * SQRT(ssq);                                              \
}                                                                                               \
                                                                                                \
/* Dot product of x[1..len) and a[1..len) (BLAS xDOT, called by reflectorApply!): four   */ \
/* interleaved partial sums (element i to sum (i-1) mod 4), combined as (s0+s1)+(s2+s3). */ \
static T P##dot4(const T *x, const T *a, i64 len)                                               \
{                                                                                               \
    T s4[4] = {0, 0, 0, 0};                                                                     \
    for (i64 i = 1; i < len; i++) s4[(i - 1) & 3] = FMA(x[i], a[i], s4[(i - 1) & 3]);          \
    return (s4[0] + s4[1]) + (s4[2] + s4[3]);                                                   \
}                                                                                               \
                                                                                                \
/* LinearAlgebra.reflector!: x[0] <- -nu, x[1:] <- x[1:]/(xi1+nu), returns tau = (xi1+nu)/nu   */ \
static T P##reflector(T *x, i64 n)                                                              \
{                                                                                               \
    if (n == 0) return 0;                                                                       \
    T xi1 = x[0];                                                                               \
    T normu = P##nrm2(x, n);                                                                    \
    if (normu == 0) return 0;                                                                   \
    T nu = COPYSIGN(normu, xi1);                                                                \
    xi1 += nu;                                                                                  \
    x[0] = -nu;                                                                                 \
    for (i64 i = 1; i < n; i++) x[i] = x[i] / xi1;                                              \
    return xi1 / nu;                                                                            \
}                                                                                               \
                                                                                                \
/* _banded_qr! (bandedqr.jl:13-28) on band storage D with bandwidths (l,u), where u already    */ \
/* includes the l padding rows added by _banded_qr (bandedqr.jl:2).  tau has min(m,n) entries; */ \
/* entries beyond ncols = min(m-1, n) are set to zero, as banded_qr!(R) allocates zeros.       */ \
int P##gbqrf(i64 m, i64 n, i64 l, i64 u, T *D, i64 ldd, T *tau)                                 \
{                                                                                               \
    if (m < 0 || n < 0 || l < 0 || u < 0 || ldd < l + u + 1) return -1;                         \
    const i64 nu_ = l + u + 1;                                                                  \
    const i64 ncols = imin(m - 1, n);                                                           \
    for (i64 k = 0; k < imin(m, n); k++) tau[k] = 0;                                            \
    for (i64 k = 0; k < ncols; k++) {                                                           \
        /* Julia k1 = k+1: x = D[u+1 : min(nu, m-k1+u+1), k1] */                                \
        i64 len = imin(nu_, m - (k + 1) + u + 1) - u;                                           \
        T *x = D + u + k * ldd;                                                                 \
        T tk = P##reflector(x, len);                                                            \
        tau[k] = tk;                                                                            \
        for (i64 j = 1; j <= imin(u, n - (k + 1)); j++) {                                       \
            T *aj = D + (u - j) + (k + j) * ldd; /* same length as x */                         \
            T vAj = tk * (aj[0] + P##dot4(x, aj, len));                                         \
            aj[0] = aj[0] - vAj;                                                                \
            for (i64 i = 1; i < len; i++) aj[i] = FMA(-vAj, x[i], aj[i]);                        \
        }                                                                                       \
    }                                                                                           \
    return 0;                                                                                   \
}                                                                                               \
                                                                                                \
/* banded_qr_lmul! (bandedqr.jl:38-94): B <- Q*B (trans='N') or Q'*B (trans='T').             */ \
/* Factors D (m x n, bandwidths (l,u)), ntau reflectors; B is m x nrhs, leading dim ldb.       */ \
int P##gbqr_lmul(char trans, i64 m, i64 n, i64 l, i64 u, const T *D, i64 ldd, const T *tau,    \
                 i64 ntau, i64 nrhs, T *B, i64 ldb)                                             \
{                                                                                               \
    int adj = (trans == 'T' || trans == 't' || trans == 'C' || trans == 'c');                   \
    const i64 kmax = imin(imin(m, n), ntau); /* colsupport(B) is all of 1:m for dense B */      \
    const i64 ilo = imax(1, -u);                                                                \
    for (i64 r = 0; r < nrhs; r++) {                                                            \
        T *bj = B + r * ldb;                                                                    \
        for (i64 t = 0; t < kmax; t++) {                                                        \
            i64 k = adj ? t : kmax - 1 - t;                                                     \
            /* bj[k] + the reflector's dot product in four interleaved partial sums  */ \
            /* (rows k+1+t, k+5+t, ...), combined (s0+s1)+(s2+s3): reflectorApply!'s  */ \
            /* dot, in the order the factorization (gbqrf) uses                        */ \
            T s4[4] = {0, 0, 0, 0};                                                             \
            for (i64 i = k + ilo; i <= imin(k + l, m - 1); i++)                                 \
                s4[(i - k - 1) & 3] = FMA(D[(i - k + u) + k * ldd], bj[i], s4[(i - k - 1) & 3]); \
            T v = tau[k] * (bj[k] + ((s4[0] + s4[1]) + (s4[2] + s4[3])));                       \
            bj[k] = bj[k] - v;                                                                  \
            for (i64 i = k + ilo; i <= imin(k + l, m - 1); i++)                                 \
                bj[i] = FMA(-D[(i - k + u) + k * ldd], v, bj[i]);                               \
        }                                                                                       \
    }                                                                                           \
    return 0;                                                                                   \
}

DEFINE_ALL(double, or_d, fma, fabs, sqrt, copysign)
DEFINE_ALL(float, or_s, fmaf, fabsf, sqrtf, copysignf)

/* Reference BLAS xTBMV (x := op(A) x, A a triangular band with k off-diagonals in BLAS
 * triangular band storage), upper/lower, 'N'/'T', unit/non-unit, incx = 1: the loop
 * order of reference DTBMV (tbmv!, src/blas.jl:71-108), each multiply-add fused. */
#define DEFINE_TBMV(T, P, FMA)                                                                  \
int P##tbmv(char uplo, char trans, char diag, i64 n, i64 k, const T *a, i64 lda, T *x)          \
{                                                                                               \
    int upper = (uplo == 'U' || uplo == 'u');                                                   \
    int notr = (trans == 'N' || trans == 'n');                                                  \
    int nounit = (diag == 'N' || diag == 'n');                                                  \
    if (n < 0) return -4;                                                                       \
    if (k < 0) return -5;                                                                       \
    if (lda < k + 1) return -7;                                                                 \
    if (n == 0) return 0;                                                                       \
    if (notr) {                                                                                 \
        if (upper) {                                                                            \
            for (i64 j = 0; j < n; j++) {                                                       \
                if (x[j] != 0) {                                                                \
                    T temp = x[j];                                                              \
                    for (i64 i = imax(0, j - k); i < j; i++)                                    \
                        x[i] = FMA(temp, a[(k - j + i) + j * lda], x[i]);                       \
                    if (nounit) x[j] = x[j] * a[k + j * lda];                                   \
                }                                                                               \
            }                                                                                   \
        } else {                                                                                \
            for (i64 j = n - 1; j >= 0; j--) {                                                  \
                if (x[j] != 0) {                                                                \
                    T temp = x[j];                                                              \
                    for (i64 i = imin(n - 1, j + k); i > j; i--)                                \
                        x[i] = FMA(temp, a[(i - j) + j * lda], x[i]);                           \
                    if (nounit) x[j] = x[j] * a[0 + j * lda];                                   \
                }                                                                               \
            }                                                                                   \
        }                                                                                       \
    } else {                                                                                    \
        if (upper) {                                                                            \
            for (i64 j = n - 1; j >= 0; j--) {                                                  \
                T temp = x[j];                                                                  \
                if (nounit) temp = temp * a[k + j * lda];                                       \
                for (i64 i = j - 1; i >= imax(0, j - k); i--)                                   \
                    temp = FMA(a[(k - j + i) + j * lda], x[i], temp);                           \
                x[j] = temp;                                                                    \
            }                                                                                   \
        } else {                                                                                \
            for (i64 j = 0; j < n; j++) {                                                       \
                T temp = x[j];                                                                  \
                if (nounit) temp = temp * a[0 + j * lda];                                       \
                for (i64 i = j + 1; i <= imin(n - 1, j + k); i++)                               \
                    temp = FMA(a[(i - j) + j * lda], x[i], temp);                               \
                x[j] = temp;                                                                    \
            }                                                                                   \
        }                                                                                       \
    }                                                                                           \
    return 0;                                                                                   \
}

DEFINE_TBMV(double, or_d, fma)
DEFINE_TBMV(float, or_s, fmaf)

/* Symmetric positive definite band: LAPACK xPBTF2 (unblocked Cholesky, the loop order of
 * dpbtf2: sqrt of the pivot, dscal of the row (upper) or column (lower) by its
 * reciprocal, dsyr rank-1 update of the trailing kn x kn triangle with each element
 * a <- fma(x_i, -x_j, a), column j skipped when x_j == 0), xPBTRS (two xTBSV sweeps)
 * and reference BLAS xSBMV (y := alpha A x + beta y, A symmetric band).  pbtrf!/pbtrs!
 * src/lapack.jl:268-332 (banded_chol!, src/symbanded/BandedCholesky.jl:2-12);
 * sbmv! src/blas.jl:35-64. */
#define DEFINE_SYMBAND(T, P, FMA, SQRT)                                                         \
int P##pbtf2(char uplo, i64 n, i64 kd, T *ab, i64 ldab, i64 *info)                             \
{                                                                                               \
    int upper = (uplo == 'U' || uplo == 'u');                                                   \
    *info = 0;                                                                                  \
    if (!upper && !(uplo == 'L' || uplo == 'l')) return -1;                                     \
    if (n < 0) return -2;                                                                       \
    if (kd < 0) return -3;                                                                      \
    if (ldab < kd + 1) return -5;                                                               \
    for (i64 j = 0; j < n; j++) {                                                               \
        T *d = ab + (upper ? kd : 0) + j * ldab;                                                \
        T ajj = *d;                                                                             \
        if (!(ajj > 0)) { *info = j + 1; return 0; }                                            \
        ajj = SQRT(ajj);                                                                        \
        *d = ajj;                                                                               \
        i64 kn = imin(kd, n - 1 - j);                                                           \
        if (kn > 0) {                                                                           \
            T r = (T)1 / ajj;                                                                   \
            /* x_t = A(j, j+t) (upper, along the row) or A(j+t, j) (lower, down the column) */   \
            for (i64 t = 1; t <= kn; t++) {                                                     \
                T *p = upper ? ab + (kd - t) + (j + t) * ldab : ab + t + j * ldab;              \
                *p = r * *p;                                                                    \
            }                                                                                   \
            for (i64 c = 1; c <= kn; c++) {                                                     \
                if (upper) {                                                                    \
                    T xc = ab[(kd - c) + (j + c) * ldab];                                       \
                    if (xc != 0) {                                                              \
                        T temp = -xc;                                                           \
                        for (i64 s = 1; s <= c; s++) {                                          \
                            T xs = ab[(kd - s) + (j + s) * ldab];                               \
                            T *a = ab + (kd + s - c) + (j + c) * ldab;                          \
                            *a = FMA(xs, temp, *a);                                             \
                        }                                                                       \
                    }                                                                           \
                } else {                                                                        \
                    T xc = ab[c + j * ldab];                                                    \
                    if (xc != 0) {                                                              \
                        T temp = -xc;                                                           \
                        for (i64 s = c; s <= kn; s++) {                                         \
                            T xs = ab[s + j * ldab];                                            \
                            T *a = ab + (s - c) + (j + c) * ldab;                               \
                            *a = FMA(xs, temp, *a);                                             \
                        }                                                                       \
                    }                                                                           \
                }                                                                               \
            }                                                                                   \
        }                                                                                       \
    }                                                                                           \
    return 0;                                                                                   \
}                                                                                               \
                                                                                                \
int P##pbtrs(char uplo, i64 n, i64 kd, i64 nrhs, const T *ab, i64 ldab, T *b, i64 ldb)         \
{                                                                                               \
    int upper = (uplo == 'U' || uplo == 'u');                                                   \
    if (!upper && !(uplo == 'L' || uplo == 'l')) return -1;                                     \
    if (n < 0) return -2;                                                                       \
    if (kd < 0) return -3;                                                                      \
    if (nrhs < 0) return -4;                                                                    \
    if (ldab < kd + 1) return -6;                                                               \
    if (ldb < imax(1, n)) return -8;                                                            \
    for (i64 r = 0; r < nrhs; r++) {                                                            \
        if (upper) {                                                                            \
            P##tbsv('U', 'T', 'N', n, kd, ab, ldab, b + r * ldb);                               \
            P##tbsv('U', 'N', 'N', n, kd, ab, ldab, b + r * ldb);                               \
        } else {                                                                                \
            P##tbsv('L', 'N', 'N', n, kd, ab, ldab, b + r * ldb);                               \
            P##tbsv('L', 'T', 'N', n, kd, ab, ldab, b + r * ldb);                               \
        }                                                                                       \
    }                                                                                           \
    return 0;                                                                                   \
}                                                                                               \
                                                                                                \
int P##sbmv(char uplo, i64 n, i64 k, T alpha, const T *a, i64 lda, const T *x, T beta, T *y)    \
{                                                                                               \
    int upper = (uplo == 'U' || uplo == 'u');                                                   \
    if (!upper && !(uplo == 'L' || uplo == 'l')) return -1;                                     \
    if (n < 0) return -2;                                                                       \
    if (k < 0) return -3;                                                                       \
    if (lda < k + 1) return -6;                                                                 \
    if (n == 0 || (alpha == 0 && beta == 1)) return 0;                                          \
    if (beta != 1)                                                                              \
        for (i64 i = 0; i < n; i++) y[i] = (beta == 0) ? (T)0 : beta * y[i];                    \
    if (alpha == 0) return 0;                                                                   \
    for (i64 j = 0; j < n; j++) {                                                               \
        T temp1 = alpha * x[j], temp2 = 0;                                                      \
        if (upper) {                                                                            \
            for (i64 i = imax(0, j - k); i < j; i++) {                                          \
                y[i] = FMA(temp1, a[(k - j + i) + j * lda], y[i]);                              \
                temp2 = FMA(a[(k - j + i) + j * lda], x[i], temp2);                             \
            }                                                                                   \
            y[j] = FMA(temp1, a[k + j * lda], y[j]);                                            \
            y[j] = FMA(alpha, temp2, y[j]);                                                     \
        } else {                                                                                \
            y[j] = FMA(temp1, a[0 + j * lda], y[j]);                                            \
            for (i64 i = j + 1; i <= imin(n - 1, j + k); i++) {                                 \
                y[i] = FMA(temp1, a[(i - j) + j * lda], y[i]);                                  \
                temp2 = FMA(a[(i - j) + j * lda], x[i], temp2);                                 \
            }                                                                                   \
            y[j] = FMA(alpha, temp2, y[j]);                                                     \
        }                                                                                       \
    }                                                                                           \
    return 0;                                                                                   \
}

DEFINE_SYMBAND(double, or_d, fma, sqrt)
DEFINE_SYMBAND(float, or_s, fmaf, sqrtf)

/* Adjoint of x = A \ b with L = w.x (the rrule of \): lambda = A^{-T} w via the
 * transposed xGBTRS on the stored factors; dL/db = lambda; dL/dA(i,j) = -lambda_i x_j on
 * the band of A (BLAS band storage, (kl+ku+1) x n, leading dim ldg). */
int or_dgb_adjoint(i64 n, i64 kl, i64 ku, const double *lu, i64 ldab, const i64 *ipiv,
                   const double *x, const double *w, double *grad_b, double *grad_band, i64 ldg)
{
    memcpy(grad_b, w, (size_t)n * sizeof(double));
    int st = or_dgbtrs('T', n, kl, ku, 1, lu, ldab, ipiv, grad_b, n > 0 ? n : 1);
    if (st) return st;
    for (i64 j = 0; j < n; j++)
        for (i64 r = 0; r < kl + ku + 1; r++) {
            i64 i = j + r - ku;
            grad_band[r + j * ldg] = (i >= 0 && i < n) ? -grad_b[i] * x[j] : 0.0;
        }
    return 0;
}

/* _gbmm! (gbmm.jl:296-340) driving an external CBLAS xGBMV through a function pointer
 * (column-major, no-transpose), so that the CPU baseline runs the reference's column loop
 * over the same OpenBLAS routine the reference ccalls, with no interpreter in the loop. */
typedef void (*cblas_dgbmv_fn)(int, int, int, int, int, int, double, const double *, int, const double *,
                               int, double, double *, int);
typedef void (*cblas_sgbmv_fn)(int, int, int, int, int, int, float, const float *, int, const float *, int,
                               float, float *, int);

#define DEFINE_PERCOL_CBLAS(T, P, FN)                                                             \
int P##gbmm_percol_cblas(void *fnp, i64 n, i64 nu, i64 m, i64 Al, i64 Au, i64 Bl, i64 Bu,         \
                         T alpha, const T *a, i64 sta, const T *b, i64 stb, T beta, T *c, i64 stc) \
{                                                                                                 \
    FN fn = (FN)fnp;                                                                              \
    const i64 Cl = Al + Bl, Cu = Au + Bu;                                                         \
    if (n == 0 || m == 0) return 0;                                                               \
    for (i64 j = 1; j <= imin(m, 1 + Bu); j++) {                                                  \
        i64 mm = imin(Cl + j, n), nn = imin(Bl + j, nu);                                          \
        if (mm > 0 && nn > 0)                                                                     \
            fn(102, 111, (int)mm, (int)nn, (int)Al, (int)Au, alpha, a, (int)sta,                  \
               b + ((j - 1) * stb + Bu - j + 1), 1, beta, c + ((j - 1) * stc + Cu - j + 1), 1);    \
    }                                                                                             \
    for (i64 j = 2 + Bu; j <= imin(imin(1 + Cu, nu + Bu), m); j++) {                              \
        i64 mm = imin(Cl + j, n), nn = imin(Bl + Bu + 1, nu - j + Bu + 1);                        \
        if (mm > 0 && nn > 0)                                                                     \
            fn(102, 111, (int)mm, (int)nn, (int)(Al + j - Bu - 1), (int)(Au - j + Bu + 1), alpha,  \
               a + (j - Bu - 1) * sta, (int)sta, b + (j - 1) * stb, 1, beta,                      \
               c + ((j - 1) * stc + Cu - j + 1), 1);                                              \
    }                                                                                             \
    for (i64 j = 2 + Cu; j <= imin(imin(m, nu + Bu), n + Cu); j++) {                              \
        i64 mm = imin(Cl + Cu + 1, n - j + Cu + 1), nn = imin(Bl + Bu + 1, nu - (j - Bu) + 1);    \
        if (mm > 0 && nn > 0)                                                                     \
            fn(102, 111, (int)mm, (int)nn, (int)(Al + Au), 0, alpha, a + (j - Bu - 1) * sta,      \
               (int)sta, b + (j - 1) * stb, 1, beta, c + (j - 1) * stc, 1);                       \
    }                                                                                             \
    for (i64 j = nu + Bu + 1; j <= imin(m, n + Cu); j++)                                          \
        for (i64 r = 0; r < Cl + Cu + 1; r++) {                                                   \
            T *p = c + (j - 1) * stc + r;                                                         \
            *p = (beta == 0) ? (T)0 : beta * *p;                                                  \
        }                                                                                         \
    return 0;                                                                                     \
}

DEFINE_PERCOL_CBLAS(double, or_d, cblas_dgbmv_fn)
DEFINE_PERCOL_CBLAS(float, or_s, cblas_sgbmv_fn)
