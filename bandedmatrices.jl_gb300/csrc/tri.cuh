// Host entry of the general triangular band solve (tri.cu): xTBSV in every uplo /
// trans / diag form with any nonzero incx, in reference DTBSV's operation order, for
// nvec vectors x + v * ldx (one warp each).
#pragma once
#include "common.cuh"

namespace bm {
template <typename T>
int tbsv_general(char uplo, char trans, char diag, i64 n, i64 k, const T* A, i64 lda, T* x, i64 incx,
                 cudaStream_t stream, const char* name, i64 nvec = 1, i64 ldx = 0);
}  // namespace bm
