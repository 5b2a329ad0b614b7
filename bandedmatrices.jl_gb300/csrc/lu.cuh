// Warp-level banded LU (xGBTF2 semantics) and solves (xGBTRS), shared by the
// single-system entry points and the batched persistent kernel.
//
// gbtrf: one warp factors one system.  The active part of the matrix at step j is
// the (kl+1) x (kl+ku+1) window A(j:j+kl, j:j+kl+ku); it lives in shared memory
// as a ring in both dimensions (logical row r <-> physical (j+r) mod (kl+1),
// logical column c <-> (j+c) mod (kl+ku+1)), so the window slides by one row
// and one column per step without moving data.  The row that enters at each
// step is fetched P steps ahead with cp.async into a staging ring.  The
// arithmetic is LAPACK's dgbtf2 operation for operation: idamax (first index of
// the largest |a|), row interchange over columns j..ju, scaling by the
// reciprocal of the pivot, and the rank-1 update a <- fma(l_i, -u_c, a) skipping
// u_c == 0 -- so factors and pivots equal the oracle's bit for bit.
//
// gbtrs: one warp sweeps one right-hand side.  The sweeps are sequential in j;
// each step's update is spread over the lanes and b is staged through shared
// memory in chunks of kChunk steps.  Every element receives its updates in the
// same order as in dgbtrs/dtbsv (the transposed triangular solve is done in
// axpy form, which preserves each element's accumulation order).  Only the
// L^T dot products of the transposed solve use a tree reduction when kl > 16.
#pragma once
#include "common.cuh"

namespace bm {

// ------------------------------------------------------------ cp.async helpers
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* src, bool valid) {
  const uint32_t d = smem_u32(dst);
  const int sz = valid ? (int)sizeof(T) : 0;
  if constexpr (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src), "r"(sz) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(sz) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Shared-memory footprint (elements of T) of one warp's gbtrf window + staging ring.
__host__ __device__ inline int lu_rs(int kl) { return (kl + 1) | 1; }  // odd column stride: no bank conflicts
template <int P>
__host__ __device__ inline i64 gbtrf_smem_elems(int kl, int ku) {
  const int K = kl + ku + 1;
  return (i64)lu_rs(kl) * K + (i64)P * K;
}

constexpr int kChunk = 32;  // solve steps staged per chunk
__host__ __device__ inline i64 gbtrs_smem_elems(int kl, int ku) {
  const int kv = kl + ku;
  // ipiv chunk (kChunk int64, as 2*kChunk T slots) + window of b (kChunk + kv + 1)
  // + chunk of L or U columns (kChunk x (kv+1))
  return 2 * kChunk + (i64)(kChunk + kv + 1) + (i64)kChunk * (kv + 1);
}

// X[s] <- X[s + d] for s in [0, count), d >= 0 (warp-cooperative, overlap-safe)
template <typename T>
__device__ __forceinline__ void warp_shift_down(T* X, int count, int d) {
  const int lane = threadIdx.x & 31;
  for (int s0 = 0; s0 < count; s0 += 32) {
    const int s = s0 + lane;
    const T v = (s < count) ? X[s + d] : T(0);
    __syncwarp();
    if (s < count) X[s] = v;
    __syncwarp();
  }
}
// X[s] <- X[s - d] for s in [d, d + count), d >= 0, processed from the top
template <typename T>
__device__ __forceinline__ void warp_shift_up(T* X, int count, int d) {
  const int lane = threadIdx.x & 31;
  for (int s0 = count - 1; s0 >= 0; s0 -= 32) {
    const int s = s0 - lane;  // relative index, descending
    const T v = (s >= 0) ? X[s] : T(0);
    __syncwarp();
    if (s >= 0) X[s + d] = v;
    __syncwarp();
  }
}

// --------------------------------------------------------------------- gbtrf
// Factors the m x n band in ab (LAPACK gbtrf storage, ldab >= 2kl+ku+1) in place;
// writes 1-based pivots to ipiv[0..min(m,n)) and returns LAPACK's info.
template <typename T, int P>
__device__ i64 gbtrf_warp(i64 m, i64 n, int kl, int ku, T* __restrict__ ab, i64 ldab, i64* __restrict__ ipiv,
                          T* __restrict__ smem) {
  const int lane = threadIdx.x & 31;
  const int kv = kl + ku, R = kl + 1, K = kv + 1, RS = lu_rs(kl);
  T* W = smem;
  T* S = smem + (i64)RS * K;
  const i64 mn = min(m, n);
  i64 info = 0;
  if (mn <= 0) return 0;

  // initial window: matrix rows 0..kl, columns 0..kv
  for (int e = lane; e < R * K; e += 32) {
    const int c = e / R, r = e - c * R;
    T v = T(0);
    if (r < m && c < n && r - c <= kl && c - r <= ku) v = ab[(kv + r - c) + (i64)c * ldab];
    W[r + c * RS] = v;
  }
  // rows kl+1 .. kl+P into the staging ring (one cp.async group per row)
  auto issue_row = [&](i64 i) {
    T* dst = S + (int)(i & (P - 1)) * K;
    for (int c = lane; c < K; c += 32) {
      const i64 col = i - kl + c;
      const bool ok = i < m && col < n;
      cp_async_elem(dst + c, ok ? ab + (kv + kl - c) + col * ldab : ab, ok);
    }
    cp_async_commit();
  };
  for (int p = 0; p < P; ++p) issue_row((i64)kl + 1 + p);
  __syncwarp();

  int pr0 = 0, pc0 = 0;
  i64 ju = 0;
  for (i64 j = 0; j < mn; ++j) {
    const int km = (int)min((i64)kl, m - 1 - j);
    // ---- pivot: first index of max |a| over logical rows 0..km of logical column 0
    T best = T(-1);
    int bidx = 0x7fffffff;
    for (int r = lane; r <= km; r += 32) {
      int pr = pr0 + r;
      pr = pr >= R ? pr - R : pr;
      const T v = fabs(W[pr + pc0 * RS]);
      if (bidx == 0x7fffffff || v > best) {
        best = v;
        bidx = r;
      }
    }
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
      const T ov = __shfl_down_sync(0xffffffffu, best, off);
      const int oi = __shfl_down_sync(0xffffffffu, bidx, off);
      if (lane + off < 32 && (ov > best || (ov == best && oi < bidx))) {
        best = ov;
        bidx = oi;
      }
    }
    const int jp = __shfl_sync(0xffffffffu, bidx, 0);
    if (lane == 0) ipiv[j] = j + jp + 1;
    int prp = pr0 + jp;
    prp = prp >= R ? prp - R : prp;
    const T piv = W[prp + pc0 * RS];
    if (piv != T(0)) {
      ju = max(ju, min(j + ku + jp, n - 1));
      const int nc = (int)(ju - j);
      if (jp != 0) {
        for (int c = lane; c <= nc; c += 32) {
          int pc = pc0 + c;
          pc = pc >= K ? pc - K : pc;
          const T t = W[pr0 + pc * RS];
          W[pr0 + pc * RS] = W[prp + pc * RS];
          W[prp + pc * RS] = t;
        }
        __syncwarp();
      }
      if (km > 0) {
        const T rcp = T(1) / piv;
        for (int r = 1 + lane; r <= km; r += 32) {
          int pr = pr0 + r;
          pr = pr >= R ? pr - R : pr;
          W[pr + pc0 * RS] = rcp * W[pr + pc0 * RS];
        }
        __syncwarp();
        for (int c = 1 + lane; c <= nc; c += 32) {
          int pc = pc0 + c;
          pc = pc >= K ? pc - K : pc;
          const T uc = W[pr0 + pc * RS];
          if (uc != T(0)) {
            const T t = -uc;
            int pr = pr0;
            for (int r = 1; r <= km; ++r) {
              pr = pr + 1 == R ? 0 : pr + 1;
              W[pr + pc * RS] = fma(W[pr + pc0 * RS], t, W[pr + pc * RS]);
            }
          }
        }
        __syncwarp();
      }
    } else if (info == 0) {
      info = j + 1;
    }
    // ---- U row j (logical row 0) and L column j are final
    const int ncw = (int)min((i64)kv, n - 1 - j);
    for (int c = lane; c <= ncw; c += 32) {
      int pc = pc0 + c;
      pc = pc >= K ? pc - K : pc;
      ab[(kv - c) + (j + c) * ldab] = W[pr0 + pc * RS];
    }
    for (int r = 1 + lane; r <= km; r += 32) {
      int pr = pr0 + r;
      pr = pr >= R ? pr - R : pr;
      ab[(kv + r) + j * ldab] = W[pr + pc0 * RS];
    }
    __syncwarp();
    if (j + 1 == mn) break;
    // ---- slide: row j+1+kl enters physical row pr0, column j+1+kv enters physical column pc0
    for (int r = lane; r < R; r += 32) W[r + pc0 * RS] = T(0);
    cp_async_wait<P - 1>();
    __syncwarp();
    const i64 inew = j + 1 + kl;
    const T* st = S + (int)(inew & (P - 1)) * K;
    for (int c = lane; c < K; c += 32) {
      int pc = pc0 + 1 + c;
      pc = pc >= K ? pc - K : pc;
      W[pr0 + pc * RS] = st[c];
    }
    __syncwarp();
    issue_row(inew + P);
    pr0 = pr0 + 1 == R ? 0 : pr0 + 1;
    pc0 = pc0 + 1 == K ? 0 : pc0 + 1;
  }
  cp_async_wait<0>();
  __syncwarp();
  return info;
}

// --------------------------------------------------------------------- gbtrs
// Solves op(A) x = b for one right-hand side b (length n, contiguous) with the
// gbtrf factors.  trans: false = 'N', true = 'T'.
template <typename T>
__device__ void gbtrs_warp(bool trans, i64 n, int kl, int ku, const T* __restrict__ ab, i64 ldab,
                           const i64* __restrict__ ipiv, T* __restrict__ b, T* __restrict__ smem) {
  const int lane = threadIdx.x & 31;
  const int kv = kl + ku;
  if (n <= 0) return;
  i64* IP = reinterpret_cast<i64*>(smem);     // kChunk pivots (8-byte aligned: smem is)
  T* X = smem + 2 * kChunk;                   // window of b: XW entries
  const int XW = kChunk + kv + 1;
  T* LC = X + XW;                             // kChunk columns x (kv+1)

  if (!trans) {
    // ---- forward: L with row interchanges (dgbtrs 'N': dswap + dger per column)
    if (kl > 0 && n > 1) {
      // X[s] = b[j0 + s]; kl entries are carried from one chunk to the next
      for (int s = lane; s < kl; s += 32) X[s] = (s < n) ? b[s] : T(0);
      for (i64 j0 = 0; j0 < n - 1; j0 += kChunk) {
        const int jn = (int)min((i64)kChunk, n - 1 - j0);
        for (int s = kl + lane; s < jn + kl; s += 32) X[s] = (j0 + s < n) ? b[j0 + s] : T(0);
        for (int e = lane; e < jn * kl; e += 32) {
          const int s = e / kl, i = e - s * kl;
          LC[s * kl + i] = (j0 + s + 1 + i < n) ? ab[(kv + 1 + i) + (j0 + s) * ldab] : T(0);
        }
        for (int s = lane; s < jn; s += 32) IP[s] = ipiv[j0 + s] - 1 - j0;
        __syncwarp();
        for (int s = 0; s < jn; ++s) {
          const int lm = (int)min((i64)kl, n - 1 - (j0 + s));
          const int l = (int)IP[s];
          if (l != s && lane == 0) {
            const T t = X[l];
            X[l] = X[s];
            X[s] = t;
          }
          __syncwarp();
          const T bj = X[s];
          if (bj != T(0)) {
            const T t = -bj;
            for (int i = lane; i < lm; i += 32) X[s + 1 + i] = fma(LC[s * kl + i], t, X[s + 1 + i]);
          }
          __syncwarp();
        }
        for (int s = lane; s < jn; s += 32) b[j0 + s] = X[s];
        __syncwarp();
        warp_shift_down(X, kl, jn);  // carry X[jn .. jn+kl) to the front
        if (j0 + jn >= n - 1)
          for (int s = lane; s < kl; s += 32)
            if (j0 + jn + s < n) b[j0 + jn + s] = X[s];
        __syncwarp();
      }
    }
    // ---- backward: U x = y (dtbsv 'U','N','N', bandwidth kv), columns n-1 .. 0
    // X[s] = b[base + s] with X[XW-1] = b[j1] at the start of each chunk
    i64 j1 = n - 1;
    i64 base = j1 - (XW - 1);
    for (int s = lane; s < XW; s += 32) X[s] = (base + s >= 0) ? b[base + s] : T(0);
    __syncwarp();
    while (true) {
      const int jn = (int)min((i64)kChunk, j1 + 1);
      // U(j-i, j) = ab[(kv-i) + j*ldab], i = 0..kv, for j = j1, j1-1, ...
      for (int e = lane; e < jn * (kv + 1); e += 32) {
        const int t = e / (kv + 1), i = e - t * (kv + 1);
        const i64 j = j1 - t;
        LC[e] = (j - i >= 0) ? ab[(kv - i) + j * ldab] : T(0);
      }
      __syncwarp();
      for (int t = 0; t < jn; ++t) {
        const i64 j = j1 - t;
        const int xs = (int)(j - base);
        const T xj = X[xs];
        if (xj != T(0)) {
          const T v = xj / LC[t * (kv + 1)];
          __syncwarp();
          if (lane == 0) X[xs] = v;
          const T tt = -v;
          const int lim = (int)min((i64)kv, j);
          for (int i = 1 + lane; i <= lim; i += 32) X[xs - i] = fma(tt, LC[t * (kv + 1) + i], X[xs - i]);
        }
        __syncwarp();
      }
      for (int t = lane; t < jn; t += 32) b[j1 - t] = X[(int)(j1 - t - base)];
      __syncwarp();
      j1 -= jn;
      if (j1 < 0) break;
      // window moves down by jn: X'[s] = X[s - jn] for s >= jn, X'[s] = b[base' + s] below
      warp_shift_up(X, XW - jn, jn);
      base -= jn;
      for (int s = lane; s < jn; s += 32) X[s] = (base + s >= 0) ? b[base + s] : T(0);
      __syncwarp();
    }
  } else {
    // ---- U^T y = b (dtbsv 'U','T','N') in axpy form: once x_i is final, x_c -= U(i,c) x_i
    for (int s = lane; s < XW; s += 32) X[s] = (s < n) ? b[s] : T(0);
    __syncwarp();
    for (i64 j0 = 0; j0 < n; j0 += kChunk) {
      const int jn = (int)min((i64)kChunk, n - j0);
      // row i of U: U(i, i+c) = ab[(kv-c) + (i+c)*ldab], c = 0..kv
      for (int e = lane; e < jn * (kv + 1); e += 32) {
        const int t = e / (kv + 1), c = e - t * (kv + 1);
        const i64 i = j0 + t;
        LC[e] = (i + c < n) ? ab[(kv - c) + (i + c) * ldab] : T(0);
      }
      __syncwarp();
      for (int t = 0; t < jn; ++t) {
        const i64 i = j0 + t;
        const T xi = X[t] / LC[t * (kv + 1)];
        __syncwarp();
        if (lane == 0) X[t] = xi;
        const int lim = (int)min((i64)kv, n - 1 - i);
        for (int c = 1 + lane; c <= lim; c += 32) X[t + c] = fma(-LC[t * (kv + 1) + c], xi, X[t + c]);
        __syncwarp();
      }
      for (int t = lane; t < jn; t += 32) b[j0 + t] = X[t];
      __syncwarp();
      // window moves up by jn
      warp_shift_down(X, XW - jn, jn);
      for (int s = XW - jn + lane; s < XW; s += 32) X[s] = (j0 + jn + s < n) ? b[j0 + jn + s] : T(0);
      __syncwarp();
    }
    // ---- L^T with interchanges, j = n-2 .. 0 (dgbtrs 'T': dgemv then dswap)
    if (kl > 0) {
      for (i64 j = n - 2; j >= 0; --j) {
        const int lm = (int)min((i64)kl, n - 1 - j);
        const T* lc = ab + (kv + 1) + j * ldab;
        T temp = T(0);
        if (kl <= 16) {
          if (lane == 0)
            for (int i = 0; i < lm; ++i) temp = fma(b[j + 1 + i], lc[i], temp);
        } else {
          for (int i = lane; i < lm; i += 32) temp = fma(b[j + 1 + i], lc[i], temp);
#pragma unroll
          for (int off = 16; off >= 1; off >>= 1) temp += __shfl_down_sync(0xffffffffu, temp, off);
        }
        if (lane == 0) {
          b[j] = fma(T(-1), temp, b[j]);
          const i64 l = ipiv[j] - 1;
          if (l != j) {
            const T t = b[l];
            b[l] = b[j];
            b[j] = t;
          }
        }
        __threadfence_block();
        __syncwarp();
      }
    }
  }
}

}  // namespace bm
