// Dense linear-algebra building blocks for the SlabLU path (FP32 / FP64).
//
// All matrices are column-major.  Pivots follow LAPACK getrf semantics with
// 0-based indices: ipiv[j] is the row interchanged with row j at step j.
//
// CTA-level routines (one thread block owns one matrix) serve the batched
// leaf and merge factorizations; the "big" kernels (one matrix spread over
// the whole GPU, host loop over panels) serve the FP64 interface blocks.
#pragma once

#include <climits>

#include <cooperative_groups.h>

#include "common.cuh"

namespace slab {

constexpr int kNT = 256;    // threads per CTA of the CTA-level routines
constexpr int kNB = 32;     // panel width
constexpr int kCT = 128;    // column tile of trailing updates
constexpr int kCTLD = kCT + 4;  // shared-memory leading dimension of a transposed tile
constexpr int kPad = 64;    // slack elements after a staged panel (micro-kernel over-read)

// ---------------------------------------------------------------------------
// Pivot search keys.  |x| is compared through its IEEE bit pattern read as an
// unsigned integer (same order as the magnitudes for non-negative values);
// NaN maps to 0, so a NaN never wins (LAPACK i?amax).  Integer compares keep
// the search off the FP64 pipe, which GB300 runs at a small fraction of the
// FP32 rate; the key has the size of T, so scratch declared as T[33] holds it.
template <typename T>
struct MagKey;
template <>
struct MagKey<double> {
  using type = unsigned long long;
  __device__ __forceinline__ static type of(double x) {
    const type b = (type)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
    return b > 0x7FF0000000000000ull ? type(0) : b;
  }
};
template <>
struct MagKey<float> {
  using type = unsigned int;
  __device__ __forceinline__ static type of(float x) {
    const type b = __float_as_uint(x) & 0x7FFFFFFFu;
    return b > 0x7F800000u ? type(0) : b;
  }
};
template <typename T>
using mag_t = typename MagKey<T>::type;
template <typename T>
__device__ __forceinline__ mag_t<T> mag_key(T x) {
  return MagKey<T>::of(x);
}

// Candidate merge with LAPACK tie-break (smallest index wins); "no candidate"
// is (0, INT_MAX), which every real candidate beats.
template <typename K>
__device__ __forceinline__ void argmax_merge(K& v, int& i, K v2, int i2) {
  if (v2 > v || (v2 == v && i2 < i)) {
    v = v2;
    i = i2;
  }
}

// Block-wide argmax over (key, index) candidates; every thread passes its
// local best and all threads get the winning index (INT_MAX if none).  sv/si
// need 33 slots (sv typed as T, reused for the keys).  Two __syncthreads.
template <typename T>
__device__ int cta_argmax(mag_t<T> v, int i, T* sv_, int* si) {
  using K = mag_t<T>;
  static_assert(sizeof(K) == sizeof(T), "key and value share scratch");
  K* sv = reinterpret_cast<K*>(sv_);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const K v2 = __shfl_down_sync(0xffffffffu, v, o);
    const int i2 = __shfl_down_sync(0xffffffffu, i, o);
    argmax_merge(v, i, v2, i2);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    sv[warp] = v;
    si[warp] = i;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    v = lane < nw ? sv[lane] : K(0);
    i = lane < nw ? si[lane] : INT_MAX;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const K v2 = __shfl_down_sync(0xffffffffu, v, o);
      const int i2 = __shfl_down_sync(0xffffffffu, i, o);
      argmax_merge(v, i, v2, i2);
    }
    if (lane == 0) si[32] = i;
  }
  __syncthreads();
  return si[32];
}

// Reciprocal of a normal double by Newton's method for 1/d, x <- x (2 - d x),
// started from the FP32 reciprocal of d's mantissa (relative error < 2^-22, so
// two steps reach the FP64 rounding level).  The exponent is handled on the bit
// pattern.  Used where a full FP64 division would sit on a latency-critical
// chain; within an ulp or two of 1/d (not correctly rounded).  Zero, subnormal,
// huge, infinite and NaN inputs take the ordinary division.
__device__ __forceinline__ double recip_newton(double d) {
  const long long b = __double_as_longlong(d);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e < 3 || e > 2044) return 1.0 / d;
  const double m = __longlong_as_double((b & 0x800FFFFFFFFFFFFFll) | (1023ll << 52));  // d / 2^(e-1023), in [1, 2)
  double x = (double)__frcp_rn((float)m);
  double r = fma(-m, x, 1.0);
  x = fma(x, r, x);
  r = fma(-m, x, 1.0);
  x = fma(x, r, x);
  // 1/d = x * 2^-(e-1023); the scale 2^(2046-e) is a normal power of two for e in [3, 2044]
  return x * __longlong_as_double((long long)(2046 - e) << 52);
}
__device__ __forceinline__ float recip_newton(float d) { return 1.0f / d; }

// 1/d computed by one thread and broadcast through shared memory (slot is a
// T in shared memory): an FP64 division is a long dependent FP64 sequence.
template <typename T>
__device__ __forceinline__ T cta_recip(T d, T* slot) {
  if (threadIdx.x == 0) *slot = T(1) / d;
  __syncthreads();
  return *slot;
}

// ---------------------------------------------------------------------------
// Unblocked LU with partial pivoting of an m x nb panel held in shared memory
// (column-major, leading dimension ldp).  piv[j] receives the panel-local row
// swapped with row j (largest magnitude, smallest index on ties, as LAPACK).
// The first exactly-zero (or NaN) pivot is recorded in *info_s as
// col_offset + j + 1 (LAPACK info); elimination continues.
// Two block barriers per column: thread t owns the rows r = t (mod blockDim),
// so the pivot search of column j+1 reads only values its own thread updated
// in column j; every warp reduces the warp candidates itself; and the
// interchange is applied inside the update from copies of the pivot row
// (prow) and of row j (orow), each nb elements of shared memory.
template <typename T>
__device__ void cta_panel_lu(T* P, int ldp, int m, int nb, int* piv, T* sv, int* si, T* prow, T* orow,
                             int* info_s, int col_offset) {
  using K = mag_t<T>;
  static_assert(sizeof(K) == sizeof(T), "key and value share scratch");
  K* wk = reinterpret_cast<K*>(sv);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (int j = 0; j < nb && j < m; ++j) {
    K best = 0;
    int bi = INT_MAX;
    for (int r = tid; r < m; r += blockDim.x) {
      if (r < j) continue;
      const K a = mag_key(P[r + j * ldp]);
      if (bi == INT_MAX || a > best) {
        best = a;
        bi = r;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const K v2 = __shfl_xor_sync(0xffffffffu, best, o);
      const int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
      argmax_merge(best, bi, v2, i2);
    }
    if (lane == 0) {
      wk[warp] = best;
      si[warp] = bi;
    }
    __syncthreads();  // (1) warp candidates; every update of column j-1 is complete
    K v = lane < nw ? wk[lane] : K(0);
    int wi = lane < nw ? si[lane] : INT_MAX;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const K v2 = __shfl_xor_sync(0xffffffffu, v, o);
      const int i2 = __shfl_xor_sync(0xffffffffu, wi, o);
      argmax_merge(v, wi, v2, i2);
    }
    const int pr = wi == INT_MAX ? j : wi;
    if (tid == 0) piv[j] = pr;
    for (int c = tid; c < nb; c += blockDim.x) {
      prow[c] = P[pr + c * ldp];
      orow[c] = P[j + c * ldp];
    }
    __syncthreads();  // (2) pivot row and row j copied
    const T d = prow[j];
    const bool ok = !(d == T(0) || d != d);
    if (!ok && tid == 0 && *info_s == 0) *info_s = col_offset + j + 1;
    for (int c = tid; c < nb; c += blockDim.x) P[j + c * ldp] = prow[c];
    if (ok) {
      const T rd = T(1) / d;
      for (int r = tid; r < m; r += blockDim.x) {
        if (r <= j) continue;
        if (r == pr) {  // receives old row j, then is eliminated like the others
          for (int c = 0; c < j; ++c) P[r + c * ldp] = orow[c];
          const T l = orow[j] * rd;
          P[r + j * ldp] = l;
          for (int c = j + 1; c < nb; ++c) P[r + c * ldp] = orow[c] - l * prow[c];
        } else {
          const T l = P[r + j * ldp] * rd;
          P[r + j * ldp] = l;
          for (int c = j + 1; c < nb; ++c) P[r + c * ldp] -= l * prow[c];
        }
      }
    } else if (pr != j) {
      for (int r = tid; r < m; r += blockDim.x)
        if (r == pr)
          for (int c = 0; c < nb; ++c) P[r + c * ldp] = orow[c];
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// C[r, c] -= sum_k A(r, k) * B(c, k) for r < mrows, c < ncols, k < kd.
// A in shared memory (element (r,k) at As[r + k*lda], lda % 4 == 0, As 16B aligned,
// readable up to 63 rows past mrows); B transposed in shared memory
// (element (c,k) at Bs[c + k*ldb], ldb % 4 == 0, readable up to 63 columns past
// ncols).  C is a generic pointer (global or shared), leading dimension ldc.
// Requires blockDim.x == 256 (16 x 16 threads, 4 x 4 outputs each).  Each
// thread loads its 16 C values before the k loop, so their latency overlaps the
// products instead of being paid once per element after it.
template <typename T>
__device__ void cta_gemm_sub(T* C, int ldc, int mrows, int ncols, const T* As, int lda, const T* Bs,
                             int ldb, int kd) {
  const int tr = threadIdx.x & 15, tc = threadIdx.x >> 4;
  for (int cb = 0; cb < ncols; cb += 64) {
    for (int rb = 0; rb < mrows; rb += 64) {
      T acc[4][4];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
      const T* ap = As + rb + 4 * tr;
      const T* bp = Bs + cb + 4 * tc;
#pragma unroll 4
      for (int kk = 0; kk < kd; ++kk) {
        const vec4<T> a = ld4(ap + kk * lda);
        const vec4<T> b = ld4(bp + kk * ldb);
        acc[0][0] += a.x * b.x; acc[0][1] += a.x * b.y; acc[0][2] += a.x * b.z; acc[0][3] += a.x * b.w;
        acc[1][0] += a.y * b.x; acc[1][1] += a.y * b.y; acc[1][2] += a.y * b.z; acc[1][3] += a.y * b.w;
        acc[2][0] += a.z * b.x; acc[2][1] += a.z * b.y; acc[2][2] += a.z * b.z; acc[2][3] += a.z * b.w;
        acc[3][0] += a.w * b.x; acc[3][1] += a.w * b.y; acc[3][2] += a.w * b.z; acc[3][3] += a.w * b.w;
      }
      T cv[4][4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = cb + 4 * tc + j;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int r = rb + 4 * tr + i;
          cv[i][j] = (c < ncols && r < mrows) ? C[r + (size_t)c * ldc] : T(0);
        }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = cb + 4 * tc + j;
        if (c >= ncols) continue;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int r = rb + 4 * tr + i;
          if (r < mrows) C[r + (size_t)c * ldc] = cv[i][j] - acc[i][j];
        }
      }
    }
  }
}

// Narrow variant of cta_gemm_sub for few columns (ncols <= 16): one thread per
// row, no wasted lanes.  Same operand layout; no over-read.  C is loaded ahead
// of the products, as in cta_gemm_sub.
template <typename T>
__device__ void cta_gemm_sub_narrow(T* C, int ldc, int mrows, int ncols, const T* As, int lda, const T* Bs,
                                    int ldb, int kd) {
  for (int r = threadIdx.x; r < mrows; r += blockDim.x) {
    T acc[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) acc[c] = T(0);
    for (int kk = 0; kk < kd; ++kk) {
      const T a = As[r + kk * lda];
#pragma unroll
      for (int c = 0; c < 16; ++c)
        if (c < ncols) acc[c] += a * Bs[c + kk * ldb];
    }
#pragma unroll
    for (int c = 0; c < 16; ++c)
      if (c < ncols) C[r + (size_t)c * ldc] -= acc[c];
  }
}

template <typename T>
__device__ __forceinline__ void cta_update(T* C, int ldc, int mrows, int ncols, const T* As, int lda, const T* Bs,
                                           int ldb, int kd) {
  if (ncols <= 16)
    cta_gemm_sub_narrow(C, ldc, mrows, ncols, As, lda, Bs, ldb, kd);
  else
    cta_gemm_sub(C, ldc, mrows, ncols, As, lda, Bs, ldb, kd);
}

// Shared-memory footprint (elements of T) of cta_getrf_aug / cta_backsub for order n.
__host__ __device__ inline int getrf_smem_elems(int n) {
  return round_up(n, 4) * kNB + kPad + kCTLD * kNB + kPad + kNB * (kNB + 1);
}

// Inverse of the unit lower-triangular nb x nb block L11 = P[0:nb, 0:nb] of a
// factored panel (P column-major, ldp), written to Ls[i + k*(kNB+1)] for the
// full kNB x kNB tile (identity outside nb, zeros above the diagonal).  Lane c
// computes column c by forward substitution, x_i = -sum_{k=c}^{i-1} L[i][k] x_k,
// with L11 first copied row-wise into Lt (kNB x (kNB+1) scratch) so that the
// lanes' reads fall in distinct banks.  Called by the 32 threads of one warp.
template <typename T>
__device__ void warp_unit_lower_inverse(const T* P, int ldp, int nb, T* Ls, T* Lt) {
  constexpr int ld = kNB + 1;
  const int lane = threadIdx.x & 31;
  for (int k = 0; k < nb; ++k)
    if (lane < nb) Lt[k + lane * ld] = P[lane + k * ldp];
  __syncwarp();
  const int c = lane;
  for (int i = 0; i < kNB; ++i) {
    T v = i == c ? T(1) : T(0);
    if (i > c && i < nb) {
      T s0 = T(0), s1 = T(0);
      int k = c;
      for (; k + 1 < i; k += 2) {
        s0 += Lt[k + i * ld] * Ls[k + c * ld];
        s1 += Lt[k + 1 + i * ld] * Ls[k + 1 + c * ld];
      }
      if (k < i) s0 += Lt[k + i * ld] * Ls[k + c * ld];
      v = -(s0 + s1);
    }
    Ls[i + c * ld] = v;
  }
  __syncwarp();
}

// U12 = L11^{-1} B in place for the nb x ct tile B held transposed in Bt
// (element (k, c) at Bt[c + k*kCTLD], ct <= kCT), with L11^{-1} from
// warp_unit_lower_inverse in Ls.  8 x 32 threads own 4 x 4 output blocks; two
// block barriers (all reads of Bt before any write).  Requires blockDim.x == 256.
template <typename T>
__device__ void cta_trmm_lower(const T* Ls, T* Bt, int nb, int ct) {
  constexpr int ld = kNB + 1;
  const int i0 = 4 * (threadIdx.x & 7), cc0 = 4 * (threadIdx.x >> 3);
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
  const int kend = min(nb, i0 + 4);
  for (int k = 0; k < kend; ++k) {
    const T l0 = Ls[i0 + k * ld], l1 = Ls[i0 + 1 + k * ld], l2 = Ls[i0 + 2 + k * ld], l3 = Ls[i0 + 3 + k * ld];
    const vec4<T> b = ld4(Bt + cc0 + k * kCTLD);
    acc[0][0] += l0 * b.x; acc[0][1] += l0 * b.y; acc[0][2] += l0 * b.z; acc[0][3] += l0 * b.w;
    acc[1][0] += l1 * b.x; acc[1][1] += l1 * b.y; acc[1][2] += l1 * b.z; acc[1][3] += l1 * b.w;
    acc[2][0] += l2 * b.x; acc[2][1] += l2 * b.y; acc[2][2] += l2 * b.z; acc[2][3] += l2 * b.w;
    acc[3][0] += l3 * b.x; acc[3][1] += l3 * b.y; acc[3][2] += l3 * b.z; acc[3][3] += l3 * b.w;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int c = cc0 + j;
    if (c >= ct) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i)
      if (i0 + i < nb) Bt[c + (i0 + i) * kCTLD] = acc[i][j];
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Blocked right-looking LU with partial pivoting of the leading n x n block of
// the column-major n x nc matrix A (global memory, lda: it is staged into
// shared memory with cp.async), applying the same row operations to all nc
// columns.  On return A[:, :n] holds L (unit, strictly lower) and U; A[:, n:]
// holds L^{-1} P A[:, n:]; ipiv[0..n) the pivots.
// *info_out = 0 or the LAPACK info of the first zero pivot.
template <typename T>
__device__ void cta_getrf_aug(T* A, int lda, int n, int nc, int* ipiv, T* smem, int* info_out) {
  __shared__ int piv_s[kNB];
  __shared__ T sv[33];
  __shared__ int si[33];
  __shared__ T prow_s[kNB];
  __shared__ T orow_s[kNB];
  __shared__ int info_s;
  const int tid = threadIdx.x;
  if (tid == 0) info_s = 0;
  T* Psm = smem;
  T* Bt = smem + round_up(n, 4) * kNB + kPad;
  T* Ls = Bt + kCTLD * kNB + kPad;  // L11^{-1} of the current panel
  for (int k0 = 0; k0 < n; k0 += kNB) {
    const int nb = min(kNB, n - k0);
    const int m = n - k0;
    const int ldq = round_up(m, 4);
    __syncthreads();
    for (int c = 0; c < nb; ++c)
      for (int r = tid; r < m; r += blockDim.x) cp_async_elem(&Psm[r + c * ldq], &A[(size_t)(k0 + c) * lda + k0 + r]);
    cp_async_wait_all();
    __syncthreads();
    cta_panel_lu(Psm, ldq, m, nb, piv_s, sv, si, prow_s, orow_s, &info_s, k0);
    if (tid < 32 && k0 + nb < nc) warp_unit_lower_inverse(Psm, ldq, nb, Ls, Bt);  // Bt is free until the tile loop
    __syncthreads();
    for (int idx = tid; idx < m * nb; idx += blockDim.x) {
      const int r = idx % m, c = idx / m;
      A[(size_t)(k0 + c) * lda + k0 + r] = Psm[r + c * ldq];
    }
    if (tid < nb) ipiv[k0 + tid] = k0 + piv_s[tid];
    // row interchanges on every column outside the panel (one thread per
    // column; a register-light loop keeps three leaves resident per SM)
    for (int c = tid; c < nc - nb; c += blockDim.x) {
      const int col = c < k0 ? c : c + nb;
      T* cp = A + (size_t)col * lda;
      for (int j = 0; j < nb; ++j) {
        const int pr = k0 + piv_s[j];
        if (pr != k0 + j) {
          T t = cp[k0 + j];
          cp[k0 + j] = cp[pr];
          cp[pr] = t;
        }
      }
    }
    __syncthreads();
    const int m2 = m - nb;
    for (int c0 = k0 + nb; c0 < nc; c0 += kCT) {
      const int ct = min(kCT, nc - c0);
      for (int idx = tid; idx < nb * ct; idx += blockDim.x) {
        const int kk = idx % nb, c = idx / nb;
        cp_async_elem(&Bt[c + kk * kCTLD], &A[(size_t)(c0 + c) * lda + k0 + kk]);
      }
      cp_async_wait_all();
      __syncthreads();
      cta_trmm_lower(Ls, Bt, nb, ct);  // U12 = L11^{-1} A12
      for (int idx = tid; idx < nb * ct; idx += blockDim.x) {
        const int kk = idx % nb, c = idx / nb;
        A[(size_t)(c0 + c) * lda + k0 + kk] = Bt[c + kk * kCTLD];
      }
      if (m2 > 0) cta_gemm_sub(A + (size_t)c0 * lda + k0 + nb, lda, m2, ct, Psm + nb, ldq, Bt, kCTLD, nb);
      __syncthreads();
    }
  }
  __syncthreads();
  if (tid == 0 && info_out) *info_out = info_s;
}

// ---------------------------------------------------------------------------
// Back substitution U X = Y in place for the nr (<= kCT) columns Y = A[:, c0 : c0+nr]
// where U is the upper triangle of A[:, :n] (global, lda; staged with cp.async).
// smem as cta_getrf_aug.
template <typename T>
__device__ void cta_backsub(T* A, int lda, int n, int c0, int nr, T* smem) {
  const int tid = threadIdx.x;
  T* Psm = smem;
  T* Bt = smem + round_up(n, 4) * kNB + kPad;
  T* Y = A + (size_t)c0 * lda;
  const int klast = ((n - 1) / kNB) * kNB;
  for (int k0 = klast; k0 >= 0; k0 -= kNB) {
    const int nb = min(kNB, n - k0);
    const int rows = k0 + nb;  // stage U[0 : k0+nb, k0 : k0+nb]
    const int ldq = round_up(rows, 4);
    __syncthreads();
    for (int c = 0; c < nb; ++c)
      for (int r = tid; r < rows; r += blockDim.x) cp_async_elem(&Psm[r + c * ldq], &A[(size_t)(k0 + c) * lda + r]);
    for (int idx = tid; idx < nb * nr; idx += blockDim.x) {
      const int kk = idx % nb, c = idx / nb;
      cp_async_elem(&Bt[c + kk * kCTLD], &Y[(size_t)c * lda + k0 + kk]);
    }
    cp_async_wait_all();
    __syncthreads();
    for (int c = tid; c < nr; c += blockDim.x) {
      for (int i = nb - 1; i >= 0; --i) {
        T s = Bt[c + i * kCTLD];
        for (int k = i + 1; k < nb; ++k) s -= Psm[k0 + i + k * ldq] * Bt[c + k * kCTLD];
        Bt[c + i * kCTLD] = s / Psm[k0 + i + i * ldq];
      }
    }
    __syncthreads();
    for (int idx = tid; idx < nb * nr; idx += blockDim.x) {
      const int kk = idx % nb, c = idx / nb;
      Y[(size_t)c * lda + k0 + kk] = Bt[c + kk * kCTLD];
    }
    if (k0 > 0) cta_update(Y, lda, k0, nr, Psm, ldq, Bt, kCTLD, nb);
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// X = U^{-1} L^{-1} P B for an n x ncols right-hand-side tile held in shared
// memory (Bsm, column-major, odd leading dimension ldbs).  LU/ipiv in global.
// Psm/Bt as for cta_getrf_aug.  lower/upper select the stages applied.
template <typename T>
__device__ void cta_getrs_smem(const T* LU, int lda, int n, const int* ipiv, T* Bsm, int ldbs, int ncols,
                               T* Psm, T* Bt, bool lower, bool upper) {
  const int tid = threadIdx.x;
  if (lower) {
    for (int c = tid; c < ncols; c += blockDim.x) {
      T* cp = Bsm + (size_t)c * ldbs;
      for (int j = 0; j < n; ++j) {
        const int pr = ipiv[j];
        if (pr != j) {
          T t = cp[j];
          cp[j] = cp[pr];
          cp[pr] = t;
        }
      }
    }
    for (int k0 = 0; k0 < n; k0 += kNB) {
      const int nb = min(kNB, n - k0);
      const int m = n - k0;
      const int ldq = round_up(m, 4);
      __syncthreads();
      for (int idx = tid; idx < m * nb; idx += blockDim.x) {
        const int r = idx % m, c = idx / m;
        Psm[r + c * ldq] = LU[(size_t)(k0 + c) * lda + k0 + r];
      }
      __syncthreads();
      for (int c = tid; c < ncols; c += blockDim.x) {
        T* cp = Bsm + (size_t)c * ldbs + k0;
        for (int i = 1; i < nb; ++i) {
          T s = cp[i];
          for (int k = 0; k < i; ++k) s -= Psm[i + k * ldq] * cp[k];
          cp[i] = s;
        }
      }
      __syncthreads();
      if (m > nb) {
        for (int idx = tid; idx < nb * ncols; idx += blockDim.x) {
          const int kk = idx % nb, c = idx / nb;
          Bt[c + kk * kCTLD] = Bsm[(size_t)c * ldbs + k0 + kk];
        }
        __syncthreads();
        cta_update(Bsm + k0 + nb, ldbs, m - nb, ncols, Psm + nb, ldq, Bt, kCTLD, nb);
      }
    }
  }
  if (upper) {
    const int klast = ((n - 1) / kNB) * kNB;
    for (int k0 = klast; k0 >= 0; k0 -= kNB) {
      const int nb = min(kNB, n - k0);
      const int rows = k0 + nb;
      const int ldq = round_up(rows, 4);
      __syncthreads();
      for (int idx = tid; idx < rows * nb; idx += blockDim.x) {
        const int r = idx % rows, c = idx / rows;
        Psm[r + c * ldq] = LU[(size_t)(k0 + c) * lda + r];
      }
      __syncthreads();
      for (int c = tid; c < ncols; c += blockDim.x) {
        T* cp = Bsm + (size_t)c * ldbs + k0;
        for (int i = nb - 1; i >= 0; --i) {
          T s = cp[i];
          for (int k = i + 1; k < nb; ++k) s -= Psm[k0 + i + k * ldq] * cp[k];
          cp[i] = s / Psm[k0 + i + i * ldq];
        }
      }
      __syncthreads();
      if (k0 > 0) {
        for (int idx = tid; idx < nb * ncols; idx += blockDim.x) {
          const int kk = idx % nb, c = idx / nb;
          Bt[c + kk * kCTLD] = Bsm[(size_t)c * ldbs + k0 + kk];
        }
        __syncthreads();
        cta_update(Bsm, ldbs, k0, ncols, Psm, ldq, Bt, kCTLD, nb);
      }
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Batched pointer arithmetic: element offsets per batch entry, or a stride.
__device__ __forceinline__ long long batch_off(const long long* off, long long stride, int b) {
  return off ? off[b] : stride * (long long)b;
}

// Batched LU of n x n matrices (nc = n) or augmented n x nc matrices.
template <typename T>
__global__ void __launch_bounds__(kNT) getrf_batched_kernel(int n, int nc, T* A, const long long* offA,
                                                           long long strideA, int lda, int* piv,
                                                           const long long* offP, long long strideP,
                                                           int* info) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int b = blockIdx.x;
  cta_getrf_aug<T>(A + batch_off(offA, strideA, b), lda, n, nc, piv + batch_off(offP, strideP, b),
                   reinterpret_cast<T*>(smem_raw), info ? info + b : nullptr);
}

// Shared-memory elements for cta_getrs_smem with an n x ncols tile.
__host__ __device__ inline int getrs_smem_elems(int n, int ncols) {
  return round_up(n, 4) * kNB + kPad + kCTLD * kNB + kPad + (n | 1) * ncols + 4;
}

// Largest column tile (multiple of 4, <= kCT) whose getrs footprint fits `bytes`.
inline int getrs_tile_cols(int n, size_t elem, size_t bytes) {
  for (int c = kCT; c >= 4; c -= 4)
    if ((size_t)getrs_smem_elems(n, c) * elem <= bytes) return c;
  return (size_t)getrs_smem_elems(n, 1) * elem <= bytes ? 1 : 0;
}

// Batched X = U^{-1} L^{-1} P B; grid (batch, column tiles).  B is n x nrhs (ldb).
template <typename T>
__global__ void __launch_bounds__(kNT) getrs_batched_kernel(int n, int nrhs, int tile, const T* LU,
                                                           const long long* offLU, long long strideLU,
                                                           int lda, const int* piv, const long long* offP,
                                                           long long strideP, T* B, const long long* offB,
                                                           long long strideB, int ldb, int lower,
                                                           int upper) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* smem = reinterpret_cast<T*>(smem_raw);
  T* Psm = smem;
  T* Bt = Psm + round_up(n, 4) * kNB + kPad;
  T* Bsm = Bt + kCTLD * kNB + kPad;
  const int ldbs = n | 1;
  const int b = blockIdx.x;
  const int c0 = blockIdx.y * tile;
  const int ncols = min(tile, nrhs - c0);
  if (ncols <= 0) return;
  T* Bg = B + batch_off(offB, strideB, b) + (size_t)c0 * ldb;
  for (int idx = threadIdx.x; idx < n * ncols; idx += blockDim.x) {
    const int r = idx % n, c = idx / n;
    Bsm[r + (size_t)c * ldbs] = Bg[r + (size_t)c * ldb];
  }
  __syncthreads();
  cta_getrs_smem<T>(LU + batch_off(offLU, strideLU, b), lda, n, piv + batch_off(offP, strideP, b), Bsm, ldbs,
                    ncols, Psm, Bt, lower != 0, upper != 0);
  for (int idx = threadIdx.x; idx < n * ncols; idx += blockDim.x) {
    const int r = idx % n, c = idx / n;
    Bg[r + (size_t)c * ldb] = Bsm[r + (size_t)c * ldbs];
  }
}

// ---------------------------------------------------------------------------
// Batched GEMM  C = beta*C + alpha * A B  (m x k times k x n), column-major.
// 64 x 64 output tile per CTA, k staged 16 at a time; grid (m/64, n/64, batch).
constexpr int kGK = 16;
constexpr int kGLD = 68;
template <typename T, bool TA = false>
__global__ void __launch_bounds__(256) gemm_kernel(int m, int n, int k, T alpha, const T* __restrict__ A,
                                                  const long long* offA, long long strideA, int lda,
                                                  const T* __restrict__ B, const long long* offB,
                                                  long long strideB, int ldb, T beta, T* C,
                                                  const long long* offC, long long strideC, int ldc) {
  __shared__ __align__(16) T As[kGK * kGLD];
  __shared__ __align__(16) T Bs[kGK * kGLD];
  const int bz = blockIdx.z;
  A += batch_off(offA, strideA, bz);
  B += batch_off(offB, strideB, bz);
  C += batch_off(offC, strideC, bz);
  const int r0 = blockIdx.x * 64, c0 = blockIdx.y * 64;
  const int tid = threadIdx.x;
  const int tr = tid & 15, tc = tid >> 4;
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
  for (int k0 = 0; k0 < k; k0 += kGK) {
    if (!TA) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int r = tid & 63, kk = (tid >> 6) + 4 * q;
        const int gr = r0 + r, gk = k0 + kk;
        As[r + kk * kGLD] = (gr < m && gk < k) ? A[gr + (size_t)gk * lda] : T(0);
      }
    } else {
      // op(A)(r, kk) = A[kk + r*lda]; consecutive threads walk kk (contiguous in A)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int kk = tid & 15, r = (tid >> 4) + 16 * q;
        const int gr = r0 + r, gk = k0 + kk;
        As[r + kk * kGLD] = (gr < m && gk < k) ? A[gk + (size_t)gr * lda] : T(0);
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int kk = tid & 15, c = (tid >> 4) + 16 * q;
      const int gc = c0 + c, gk = k0 + kk;
      Bs[c + kk * kGLD] = (gc < n && gk < k) ? B[gk + (size_t)gc * ldb] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kGK; ++kk) {
      const vec4<T> a = ld4(As + 4 * tr + kk * kGLD);
      const vec4<T> b = ld4(Bs + 4 * tc + kk * kGLD);
      acc[0][0] += a.x * b.x; acc[0][1] += a.x * b.y; acc[0][2] += a.x * b.z; acc[0][3] += a.x * b.w;
      acc[1][0] += a.y * b.x; acc[1][1] += a.y * b.y; acc[1][2] += a.y * b.z; acc[1][3] += a.y * b.w;
      acc[2][0] += a.z * b.x; acc[2][1] += a.z * b.y; acc[2][2] += a.z * b.z; acc[2][3] += a.z * b.w;
      acc[3][0] += a.w * b.x; acc[3][1] += a.w * b.y; acc[3][2] += a.w * b.z; acc[3][3] += a.w * b.w;
    }
    __syncthreads();
  }
  // every C load of the thread is issued before any store (one latency, not 16)
  T cv[4][4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int c = c0 + 4 * tc + j;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = r0 + 4 * tr + i;
      cv[i][j] = (beta != T(0) && c < n && r < m) ? C[r + (size_t)c * ldc] : T(0);
    }
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int c = c0 + 4 * tc + j;
    if (c >= n) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = r0 + 4 * tr + i;
      if (r >= m) continue;
      C[r + (size_t)c * ldc] = (beta == T(0) ? T(0) : beta * cv[i][j]) + alpha * acc[i][j];
    }
  }
}

// Same product with 32 x 32 output tiles (2 x 2 outputs per thread), for FP64
// shapes whose 64 x 64 grid would leave SMs idle: GB300 retires about two FP64
// FMAs per clock per SM, so FP64 products want every SM busy.
template <typename T>
__global__ void __launch_bounds__(256) gemm32_kernel(int m, int n, int k, T alpha, const T* __restrict__ A,
                                                    const long long* offA, long long strideA, int lda,
                                                    const T* __restrict__ B, const long long* offB,
                                                    long long strideB, int ldb, T beta, T* C,
                                                    const long long* offC, long long strideC, int ldc) {
  constexpr int kLD = 34;
  __shared__ __align__(16) T As[kGK * kLD];
  __shared__ __align__(16) T Bs[kGK * kLD];
  const int bz = blockIdx.z;
  A += batch_off(offA, strideA, bz);
  B += batch_off(offB, strideB, bz);
  C += batch_off(offC, strideC, bz);
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  const int tid = threadIdx.x;
  const int tr = tid & 15, tc = tid >> 4;
  T acc[2][2] = {{T(0), T(0)}, {T(0), T(0)}};
  for (int k0 = 0; k0 < k; k0 += kGK) {
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int idx = tid + 256 * q;  // 512 elements of each tile
      const int r = idx & 31, kk = idx >> 5;
      const int gr = r0 + r, gk = k0 + kk;
      As[r + kk * kLD] = (gr < m && gk < k) ? A[gr + (size_t)gk * lda] : T(0);
      const int kb = idx & 15, c = idx >> 4;
      const int gc = c0 + c, gkb = k0 + kb;
      Bs[c + kb * kLD] = (gc < n && gkb < k) ? B[gkb + (size_t)gc * ldb] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kGK; ++kk) {
      const T a0 = As[2 * tr + kk * kLD], a1 = As[2 * tr + 1 + kk * kLD];
      const T b0 = Bs[2 * tc + kk * kLD], b1 = Bs[2 * tc + 1 + kk * kLD];
      acc[0][0] += a0 * b0;
      acc[0][1] += a0 * b1;
      acc[1][0] += a1 * b0;
      acc[1][1] += a1 * b1;
    }
    __syncthreads();
  }
  T cv[2][2];
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const int c = c0 + 2 * tc + j;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int r = r0 + 2 * tr + i;
      cv[i][j] = (beta != T(0) && c < n && r < m) ? C[r + (size_t)c * ldc] : T(0);
    }
  }
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const int c = c0 + 2 * tc + j;
    if (c >= n) continue;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int r = r0 + 2 * tr + i;
      if (r >= m) continue;
      C[r + (size_t)c * ldc] = (beta == T(0) ? T(0) : beta * cv[i][j]) + alpha * acc[i][j];
    }
  }
}

// Narrow GEMM (n <= NC columns): one thread per row of C, B staged in shared
// memory; reads A once (memory-bound shape of the solve phase).
// grid (ceil(m/256), 1, batch).
template <typename T, int NC>
__global__ void __launch_bounds__(256) gemm_narrow_kernel(int m, int n, int k, T alpha, const T* __restrict__ A,
                                                         const long long* offA, long long strideA, int lda,
                                                         const T* __restrict__ B, const long long* offB,
                                                         long long strideB, int ldb, T beta, T* C,
                                                         const long long* offC, long long strideC, int ldc) {
  constexpr int KC = 128;
  __shared__ T Bs[KC * NC];
  const int bz = blockIdx.z;
  A += batch_off(offA, strideA, bz);
  B += batch_off(offB, strideB, bz);
  C += batch_off(offC, strideC, bz);
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  T acc[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) acc[c] = T(0);
  for (int k0 = 0; k0 < k; k0 += KC) {
    const int kc = min(KC, k - k0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < KC * NC; idx += blockDim.x) {
      const int kk = idx % KC, c = idx / KC;
      Bs[c * KC + kk] = (kk < kc && c < n) ? B[(k0 + kk) + (size_t)c * ldb] : T(0);
    }
    __syncthreads();
    if (r < m) {
      const T* ap = A + r + (size_t)k0 * lda;
      int kk = 0;
      // eight loads of A in flight before their products (same order of the sums)
      for (; kk + 8 <= kc; kk += 8) {
        T av[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) av[u] = ap[(size_t)(kk + u) * lda];
#pragma unroll
        for (int u = 0; u < 8; ++u)
#pragma unroll
          for (int c = 0; c < NC; ++c) acc[c] += av[u] * Bs[c * KC + kk + u];
      }
      for (; kk < kc; ++kk) {
        const T a = ap[(size_t)kk * lda];
#pragma unroll
        for (int c = 0; c < NC; ++c) acc[c] += a * Bs[c * KC + kk];
      }
    }
  }
  if (r < m) {
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      if (c >= n) break;
      T* cp = C + r + (size_t)c * ldc;
      *cp = (beta == T(0) ? T(0) : beta * *cp) + alpha * acc[c];
    }
  }
}

// The same product for grids of few CTAs: 32 rows per CTA, k split over the 8
// warps (warp w takes k = w, w+8, ...; each load is one coalesced 32-row
// segment of a column of A), partial sums reduced in a fixed order through
// shared memory (deterministic).  grid (ceil(m/32), 1, batch).
template <typename T, int NC>
__global__ void __launch_bounds__(256) gemm_narrow_ks_kernel(int m, int n, int k, T alpha, const T* __restrict__ A,
                                                            const long long* offA, long long strideA, int lda,
                                                            const T* __restrict__ B, const long long* offB,
                                                            long long strideB, int ldb, T beta, T* C,
                                                            const long long* offC, long long strideC, int ldc) {
  constexpr int KC = 256, KG = 8;
  __shared__ T Bs[KC * NC];  // B chunk; then the warps' partial sums (KG x 32 x NC <= KC x NC)
  const int bz = blockIdx.z;
  A += batch_off(offA, strideA, bz);
  B += batch_off(offB, strideB, bz);
  C += batch_off(offC, strideC, bz);
  const int lr = threadIdx.x & 31, kg = threadIdx.x >> 5;
  const int r = blockIdx.x * 32 + lr;
  T acc[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) acc[c] = T(0);
  for (int k0 = 0; k0 < k; k0 += KC) {
    const int kc = min(KC, k - k0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < KC * NC; idx += blockDim.x) {
      const int kk = idx % KC, c = idx / KC;
      Bs[c * KC + kk] = (kk < kc && c < n) ? B[(k0 + kk) + (size_t)c * ldb] : T(0);
    }
    __syncthreads();
    if (r < m) {
      const T* ap = A + r + (size_t)k0 * lda;
#pragma unroll 4
      for (int kk = kg; kk < kc; kk += KG) {
        const T a = ap[(size_t)kk * lda];
#pragma unroll
        for (int c = 0; c < NC; ++c) acc[c] += a * Bs[c * KC + kk];
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int c = 0; c < NC; ++c) Bs[(kg * 32 + lr) * NC + c] = acc[c];
  __syncthreads();
  if (kg == 0 && r < m) {
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      if (c >= n) break;
      T sum = Bs[lr * NC + c];
      for (int w = 1; w < KG; ++w) sum += Bs[(w * 32 + lr) * NC + c];
      T* cp = C + r + (size_t)c * ldc;
      *cp = (beta == T(0) ? T(0) : beta * *cp) + alpha * sum;
    }
  }
}

// ---------------------------------------------------------------------------
// Batched ipiv -> row permutation (perm[i] = source row of row i), one thread
// per matrix.
__global__ void perm_batched_kernel(const int* ipiv, long long strideP, int n, int batch, int* perm,
                                    long long strideQ);

// Warp-per-matrix X = U^{-1} L^{-1} P B for few right-hand sides (nrhs <= 4):
// one warp per batch entry, 8 warps per CTA, the vector in shared memory.
constexpr int kWarpSolveWarps = 8;
constexpr int kWarpSlots = 16;  // rows per lane: n <= 512

// Warp-per-matrix X = A^{-T} B = P^T L^{-T} U^{-T} B (nrhs <= 4): dot-product
// substitution along the columns of U (forward with U^T) and of L (backward
// with L^T); each column segment is read by the 32 lanes (coalesced) and
// reduced with shuffles; the next column is prefetched.
template <typename T>
__global__ void __launch_bounds__(32 * kWarpSolveWarps)
    getrs_warp_t_kernel(int n, int nrhs, const T* __restrict__ LU, const long long* offLU, long long strideLU,
                        int lda, const int* __restrict__ perm, const long long* offP, long long strideP, T* B,
                        const long long* offB, long long strideB, int ldb, int batch) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int b = blockIdx.x * kWarpSolveWarps + warp;
  if (b >= batch) return;
  T* xs = reinterpret_cast<T*>(smem_raw) + (size_t)warp * n * nrhs;
  const T* __restrict__ A = LU + batch_off(offLU, strideLU, b);
  const int* pv = perm + batch_off(offP, strideP, b);
  T* Bg = B + batch_off(offB, strideB, b);
  for (int c = 0; c < nrhs; ++c)
    for (int i = lane; i < n; i += 32) xs[i + c * n] = Bg[i + (size_t)c * ldb];
  __syncwarp();
  T cur[kWarpSlots], nxt[kWarpSlots];
  // forward with U^T: x_k = (b_k - U[0:k, k] . x[0:k]) / U[k, k]
#pragma unroll
  for (int t = 0; t < kWarpSlots; ++t) cur[t] = T(0);
  for (int k = 0; k < n; ++k) {
    if (k + 1 < n) {
      const T* nc = A + (size_t)(k + 1) * lda;
#pragma unroll
      for (int t = 0; t < kWarpSlots; ++t) {
        const int i = lane + 32 * t;
        nxt[t] = i <= k + 1 ? nc[i] : T(0);  // U[0:k+1, k+1] and the diagonal
      }
    }
    const T* ck = A + (size_t)k * lda;
    const T d = ck[k];
    for (int c = 0; c < nrhs; ++c) {
      T part = T(0);
#pragma unroll
      for (int t = 0; t < kWarpSlots; ++t) {
        const int i = lane + 32 * t;
        if (i < k) part += (k == 0 ? T(0) : cur[t]) * xs[i + c * n];
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
      const T xk = (xs[k + c * n] - part) / d;
      __syncwarp();
      if (lane == 0) xs[k + c * n] = xk;
      __syncwarp();
    }
#pragma unroll
    for (int t = 0; t < kWarpSlots; ++t) cur[t] = nxt[t];
  }
  // backward with L^T (unit): x_k = b_k - L[k+1:n, k] . x[k+1:n]
  {
    const T* cc = A + (size_t)(n - 1) * lda;
#pragma unroll
    for (int t = 0; t < kWarpSlots; ++t) {
      const int i = lane + 32 * t;
      cur[t] = (i > n - 1 && i < n) ? cc[i] : T(0);
    }
  }
  for (int k = n - 1; k >= 0; --k) {
    if (k > 0) {
      const T* nc = A + (size_t)(k - 1) * lda;
#pragma unroll
      for (int t = 0; t < kWarpSlots; ++t) {
        const int i = lane + 32 * t;
        nxt[t] = (i > k - 1 && i < n) ? nc[i] : T(0);
      }
    }
    for (int c = 0; c < nrhs; ++c) {
      T part = T(0);
#pragma unroll
      for (int t = 0; t < kWarpSlots; ++t) {
        const int i = lane + 32 * t;
        if (i > k && i < n) part += cur[t] * xs[i + c * n];
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
      const T xk = xs[k + c * n] - part;
      __syncwarp();
      if (lane == 0) xs[k + c * n] = xk;
      __syncwarp();
    }
#pragma unroll
    for (int t = 0; t < kWarpSlots; ++t) cur[t] = nxt[t];
  }
  // x = P^T z: row perm[i] of x is row i of z
  for (int c = 0; c < nrhs; ++c)
    for (int i = lane; i < n; i += 32) Bg[pv[i] + (size_t)c * ldb] = xs[i + c * n];
}

// Blocked warp-per-matrix solve (NR = nrhs <= 4, n <= 32 * kWarpSlots), in the
// elimination order of an unblocked substitution: rows in blocks of 32.
// The diagonal triangle of a block is solved with one lane per row (the
// block's solution stays in registers and is broadcast by shuffles), and the
// update of the other rows runs one 32-row group at a time over all 32
// columns of the block, so each lane has 32 independent loads of the factor in
// flight: about n^2 / 2048 memory round trips per pass instead of n.
// g0 / ng: this warp takes the row groups g0, g0 + ng, ... (the CTA variant
// spreads them over its warps).
template <typename T, int NR>
__device__ __forceinline__ void warp_block_update(const T* __restrict__ A, int lda, int kb, int nb, int rbeg, int rend,
                                                  const T (&x)[NR], T* xs, int n, int lane, int g0 = 0, int ng = 1) {
#pragma unroll 1
  for (int r = rbeg + 32 * g0 + lane; r - lane < rend; r += 32 * ng) {
    const bool ok = r < rend;
    T a[32];
    const T* pc = A + (size_t)kb * lda + (ok ? r : 0);
#pragma unroll
    for (int k = 0; k < 32; ++k) {
      a[k] = (ok && k < nb) ? *pc : T(0);
      pc += lda;
    }
    T acc[NR];
#pragma unroll
    for (int c = 0; c < NR; ++c) acc[c] = T(0);
#pragma unroll
    for (int k = 0; k < 32; ++k)
#pragma unroll
      for (int c = 0; c < NR; ++c) acc[c] += a[k] * __shfl_sync(0xffffffffu, x[c], k);
    if (ok)
#pragma unroll
      for (int c = 0; c < NR; ++c) xs[r + c * n] -= acc[c];
  }
}

template <typename T, int NR>
__global__ void __launch_bounds__(32 * kWarpSolveWarps)
    getrs_warp_blocked_kernel(int n, const T* __restrict__ LU, const long long* offLU, long long strideLU, int lda,
                              const int* __restrict__ perm, const long long* offP, long long strideP, T* B,
                              const long long* offB, long long strideB, int ldb, int batch) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int b = blockIdx.x * kWarpSolveWarps + warp;
  if (b >= batch) return;
  T* xs = reinterpret_cast<T*>(smem_raw) + (size_t)warp * n * NR;
  const T* __restrict__ A = LU + batch_off(offLU, strideLU, b);
  const int* pv = perm + batch_off(offP, strideP, b);
  T* Bg = B + batch_off(offB, strideB, b);
  for (int c = 0; c < NR; ++c)
    for (int i = lane; i < n; i += 32) xs[i + c * n] = Bg[pv[i] + (size_t)c * ldb];
  __syncwarp();
  // forward, unit lower
  for (int kb = 0; kb < n; kb += 32) {
    const int nb = min(32, n - kb);
    T x[NR];
#pragma unroll
    for (int c = 0; c < NR; ++c) x[c] = lane < nb ? xs[kb + lane + c * n] : T(0);
    {
      T lrow[32];
      const T* pc = A + (size_t)kb * lda + kb + (lane < nb ? lane : 0);
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        lrow[k] = (k < lane && lane < nb) ? *pc : T(0);
        pc += lda;
      }
#pragma unroll
      for (int k = 0; k < 31; ++k)
#pragma unroll
        for (int c = 0; c < NR; ++c) x[c] -= lrow[k] * __shfl_sync(0xffffffffu, x[c], k);
    }
#pragma unroll
    for (int c = 0; c < NR; ++c)
      if (lane < nb) xs[kb + lane + c * n] = x[c];
    warp_block_update<T, NR>(A, lda, kb, nb, kb + nb, n, x, xs, n, lane);
    __syncwarp();
  }
  // backward, upper (non-unit)
  for (int kb = ((n - 1) / 32) * 32; kb >= 0; kb -= 32) {
    const int nb = min(32, n - kb);
    T x[NR];
#pragma unroll
    for (int c = 0; c < NR; ++c) x[c] = lane < nb ? xs[kb + lane + c * n] : T(0);
    {
      T urow[32];
      const T* pc = A + (size_t)kb * lda + kb + (lane < nb ? lane : 0);
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        urow[k] = (k > lane && k < nb) ? *pc : T(0);
        pc += lda;
      }
      const T d = lane < nb ? A[(kb + lane) + (size_t)(kb + lane) * lda] : T(1);
#pragma unroll
      for (int k = 31; k >= 0; --k) {
        if (k >= nb) continue;
#pragma unroll
        for (int c = 0; c < NR; ++c) {
          if (lane == k) x[c] = x[c] / d;
          x[c] -= urow[k] * __shfl_sync(0xffffffffu, x[c], k);
        }
      }
    }
#pragma unroll
    for (int c = 0; c < NR; ++c)
      if (lane < nb) xs[kb + lane + c * n] = x[c];
    warp_block_update<T, NR>(A, lda, kb, nb, 0, kb, x, xs, n, lane);
    __syncwarp();
  }
  for (int c = 0; c < NR; ++c)
    for (int i = lane; i < n; i += 32) Bg[i + (size_t)c * ldb] = xs[i + c * n];
}

// The same solve with one CTA per matrix, for batches of few large matrices
// (the top merge levels): warp 0 solves each diagonal 32-row triangle as the
// warp kernel does, then all warps update the rows below (above) it, 32-row
// groups spread over the warps, with a block barrier around each update.  Each
// row sees the same operations in the same order as in the warp kernel.
template <typename T, int NR>
__global__ void __launch_bounds__(256)
    getrs_cta_blocked_kernel(int n, const T* __restrict__ LU, const long long* offLU, long long strideLU, int lda,
                             const int* __restrict__ perm, const long long* offP, long long strideP, T* B,
                             const long long* offB, long long strideB, int ldb, int batch) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int b = blockIdx.x;
  if (b >= batch) return;
  T* xs = reinterpret_cast<T*>(smem_raw);
  const T* __restrict__ A = LU + batch_off(offLU, strideLU, b);
  const int* pv = perm + batch_off(offP, strideP, b);
  T* Bg = B + batch_off(offB, strideB, b);
  for (int c = 0; c < NR; ++c)
    for (int i = threadIdx.x; i < n; i += blockDim.x) xs[i + c * n] = Bg[pv[i] + (size_t)c * ldb];
  __syncthreads();
  // forward, unit lower
  for (int kb = 0; kb < n; kb += 32) {
    const int nb = min(32, n - kb);
    if (warp == 0) {
      T x[NR];
#pragma unroll
      for (int c = 0; c < NR; ++c) x[c] = lane < nb ? xs[kb + lane + c * n] : T(0);
      T lrow[32];
      const T* pc = A + (size_t)kb * lda + kb + (lane < nb ? lane : 0);
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        lrow[k] = (k < lane && lane < nb) ? *pc : T(0);
        pc += lda;
      }
#pragma unroll
      for (int k = 0; k < 31; ++k)
#pragma unroll
        for (int c = 0; c < NR; ++c) x[c] -= lrow[k] * __shfl_sync(0xffffffffu, x[c], k);
#pragma unroll
      for (int c = 0; c < NR; ++c)
        if (lane < nb) xs[kb + lane + c * n] = x[c];
    }
    __syncthreads();
    T x[NR];
#pragma unroll
    for (int c = 0; c < NR; ++c) x[c] = lane < nb ? xs[kb + lane + c * n] : T(0);
    warp_block_update<T, NR>(A, lda, kb, nb, kb + nb, n, x, xs, n, lane, warp, nw);
    __syncthreads();
  }
  // backward, upper (non-unit)
  for (int kb = ((n - 1) / 32) * 32; kb >= 0; kb -= 32) {
    const int nb = min(32, n - kb);
    if (warp == 0) {
      T x[NR];
#pragma unroll
      for (int c = 0; c < NR; ++c) x[c] = lane < nb ? xs[kb + lane + c * n] : T(0);
      T urow[32];
      const T* pc = A + (size_t)kb * lda + kb + (lane < nb ? lane : 0);
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        urow[k] = (k > lane && k < nb) ? *pc : T(0);
        pc += lda;
      }
      const T d = lane < nb ? A[(kb + lane) + (size_t)(kb + lane) * lda] : T(1);
#pragma unroll
      for (int k = 31; k >= 0; --k) {
        if (k >= nb) continue;
#pragma unroll
        for (int c = 0; c < NR; ++c) {
          if (lane == k) x[c] = x[c] / d;
          x[c] -= urow[k] * __shfl_sync(0xffffffffu, x[c], k);
        }
      }
#pragma unroll
      for (int c = 0; c < NR; ++c)
        if (lane < nb) xs[kb + lane + c * n] = x[c];
    }
    __syncthreads();
    T x[NR];
#pragma unroll
    for (int c = 0; c < NR; ++c) x[c] = lane < nb ? xs[kb + lane + c * n] : T(0);
    warp_block_update<T, NR>(A, lda, kb, nb, 0, kb, x, xs, n, lane, warp, nw);
    __syncthreads();
  }
  for (int c = 0; c < NR; ++c)
    for (int i = threadIdx.x; i < n; i += blockDim.x) Bg[i + (size_t)c * ldb] = xs[i + c * n];
}

// Batched X = U^{-1} L^{-1} P B for many right-hand sides (the solve phase with
// more than four columns): one CTA per (matrix, 32-column tile) with the tile in
// shared memory.  Per 32-row block the diagonal triangle is solved by lane-per-
// row substitution with shuffles (each warp four columns, the triangle's rows
// in registers), then the rows beyond it are updated: the block's factor rows
// are staged in shared memory 128 rows at a time and each thread keeps one
// column of the solved block in registers, so an update is four FMAs per
// shared-memory load.  perm from build_perm_batched.  grid (batch, tiles).
constexpr int kManyCols = 32;
constexpr int kManyMaxN = 1024;  // the tile of n rows stays in shared memory
constexpr int kManyChunk = 128;
// FP32: registers capped for three resident CTAs per SM (80, a few spilled
// bytes outside the update loop), measured faster than two (94 registers) and
// four (64, more spills)
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 1) getrs_many_kernel(int n, int nrhs, const T* __restrict__ LU,
                                                         long long strideLU, int lda, const int* __restrict__ perm,
                                                         long long strideP, T* B, long long strideB, int ldb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int NC = kManyCols, CH = kManyChunk;
  const int ldx = n | 1;
  T* Xs = reinterpret_cast<T*>(smem_raw);            // n x NC, ld n|1
  constexpr int LS = 36;                              // Ls row stride: rows start 16-byte aligned
  T* Ls = Xs + (((size_t)ldx * NC + 3) & ~(size_t)3);  // CH x LS: staged factor rows, 16-byte aligned
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int b = blockIdx.x;
  const int c0 = blockIdx.y * NC;
  const int nc = min(NC, nrhs - c0);
  const T* A = LU + strideLU * b;
  const int* pv = perm + strideP * b;
  T* Bg = B + strideB * b + (size_t)c0 * ldb;
  // loads are issued eight at a time before their stores (one memory latency per
  // eight elements)
  for (int base = tid; base < n * NC; base += 8 * blockDim.x) {
    T v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = base + u * blockDim.x;
      const int r = idx % n, c = idx / n;
      v[u] = (idx < n * NC && c < nc) ? Bg[pv[r] + (size_t)c * ldb] : T(0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = base + u * blockDim.x;
      if (idx < n * NC) Xs[(idx % n) + (idx / n) * ldx] = v[u];
    }
  }
  __syncthreads();
  const int col = tid % NC, rph = tid / NC;  // update: this thread's column and row phase (8 phases)
  for (int pass = 0; pass < 2; ++pass) {
    const bool fwd = pass == 0;
    const int nblk = (n + 31) / 32;
    for (int st = 0; st < nblk; ++st) {
      const int kb = fwd ? st * 32 : (nblk - 1 - st) * 32;
      const int nb = min(32, n - kb);
      // (a) diagonal triangle: warp w solves columns 4w .. 4w+3
      {
        T lrow[32];
        const T* pc = A + (size_t)kb * lda + kb + (lane < nb ? lane : 0);
#pragma unroll
        for (int k = 0; k < 32; ++k) {
          lrow[k] = (lane < nb && k < nb && (fwd ? k < lane : k > lane)) ? *pc : T(0);
          pc += lda;
        }
        // the diagonal's reciprocal, once per lane (this is the solve phase: a
        // product with 1/d instead of the quotient changes only the last bit)
        const T rd = T(1) / ((!fwd && lane < nb) ? A[(kb + lane) + (size_t)(kb + lane) * lda] : T(1));
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int c = 4 * warp + q;
          T x = lane < nb ? Xs[kb + lane + c * ldx] : T(0);
          if (fwd) {
#pragma unroll
            for (int k = 0; k < 31; ++k) x -= lrow[k] * __shfl_sync(0xffffffffu, x, k);
          } else {
#pragma unroll
            for (int k = 31; k >= 0; --k) {
              if (k >= nb) continue;
              if (lane == k) x *= rd;
              x -= lrow[k] * __shfl_sync(0xffffffffu, x, k);
            }
          }
          if (lane < nb) Xs[kb + lane + c * ldx] = x;
        }
      }
      __syncthreads();
      // (b) the other rows: below the block (forward) or above it (backward)
      const int rlo = fwd ? kb + nb : 0, rhi = fwd ? n : kb;
      T xj[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) xj[k] = k < nb ? Xs[kb + k + col * ldx] : T(0);
      for (int r0 = rlo; r0 < rhi; r0 += CH) {
        const int rc = min(CH, rhi - r0);
        for (int base = tid; base < rc * 32; base += 8 * blockDim.x) {
          T v[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int idx = base + u * blockDim.x;
            const int rr = idx % rc, k = idx / rc;
            v[u] = (idx < rc * 32 && k < nb) ? A[(r0 + rr) + (size_t)(kb + k) * lda] : T(0);
          }
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int idx = base + u * blockDim.x;
            if (idx < rc * 32) Ls[(idx % rc) * LS + idx / rc] = v[u];
          }
        }
        __syncthreads();
        for (int rr = rph; rr < rc; rr += 256 / NC) {
          T acc = Xs[r0 + rr + col * ldx];
          const T* lr = Ls + rr * LS;
#pragma unroll
          for (int k = 0; k < 32; k += 4) {
            const vec4<T> l4 = ld4(lr + k);  // one shared-memory load for four FMAs
            acc -= l4.x * xj[k];
            acc -= l4.y * xj[k + 1];
            acc -= l4.z * xj[k + 2];
            acc -= l4.w * xj[k + 3];
          }
          Xs[r0 + rr + col * ldx] = acc;
        }
        __syncthreads();
      }
    }
  }
  for (int idx = tid; idx < n * nc; idx += blockDim.x) {
    const int r = idx % n, c = idx / n;
    Bg[r + (size_t)c * ldb] = Xs[r + c * ldx];
  }
}

__host__ __device__ inline size_t getrs_many_smem_bytes(int n, size_t elem) {
  // Xs, then Ls on a 16-byte boundary (4 spare elements)
  return ((size_t)(n | 1) * kManyCols + 4 + (size_t)kManyChunk * 36) * elem;
}

// Cooperative triangular solves with one large factored matrix (FP64
// interface blocks): X = U^{-1} L^{-1} P B for nrhs <= 8 columns, using the
// precomputed inverses of the bs x bs diagonal triangles (tri_inv_blocks).
// CTA j owns the row blocks j, j+G, ... (at most kCoopMaxOwn); per block b
// its owner forms x_b = inv_b acc_b, then after one grid-wide barrier every
// CTA subtracts the block's contribution from the rows it owns.
constexpr int kCoopMaxRhs = 8;
constexpr int kCoopMaxOwn = 4;

// Transposed copy: dst(r, k) = src[r * lds + k] for an rb x kb result.
template <typename T>
__device__ __forceinline__ void stage_block_t(T* dst, int ldd, const T* src, int lds, int rb, int kb) {
  constexpr int kPer = 16;
  const int tot = rb * kb;
  for (int base = 0; base < tot; base += kPer * blockDim.x) {
    T v[kPer];
#pragma unroll
    for (int t = 0; t < kPer; ++t) {
      const int idx = base + t * blockDim.x + threadIdx.x;
      v[t] = idx < tot ? src[(size_t)(idx / kb) * lds + (idx % kb)] : T(0);  // contiguous in k
    }
#pragma unroll
    for (int t = 0; t < kPer; ++t) {
      const int idx = base + t * blockDim.x + threadIdx.x;
      if (idx < tot) dst[(idx / kb) + (idx % kb) * ldd] = v[t];
    }
  }
}

// Copy an rb x kb column-major block (ld lds) into shared memory (ld ldd) with
// every load of a thread issued before its stores (one memory round trip).
template <typename T>
__device__ __forceinline__ void stage_block(T* dst, int ldd, const T* src, int lds, int rb, int kb) {
  constexpr int kPer = 16;  // 64 x 64 / 256 threads
  const int tot = rb * kb;
  for (int base = 0; base < tot; base += kPer * blockDim.x) {
    T v[kPer];
#pragma unroll
    for (int t = 0; t < kPer; ++t) {
      const int idx = base + t * blockDim.x + threadIdx.x;
      v[t] = idx < tot ? src[(size_t)(idx / rb) * lds + (idx % rb)] : T(0);
    }
#pragma unroll
    for (int t = 0; t < kPer; ++t) {
      const int idx = base + t * blockDim.x + threadIdx.x;
      if (idx < tot) dst[(idx % rb) + (idx / rb) * ldd] = v[t];
    }
  }
}
template <typename T>
__global__ void __launch_bounds__(256) trsv_coop_kernel(const T* __restrict__ LU, int lda, int n,
                                                       const int* __restrict__ perm, const T* __restrict__ Linv,
                                                       const T* __restrict__ Uinv, int bs,
                                                       const T* __restrict__ Bin, int ldb, T* X, int ldx, int nrhs,
                                                       int trans) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ldd = bs + 1;
  T* acc = reinterpret_cast<T*>(smem_raw);          // kCoopMaxOwn x (bs x nrhs)
  T* dblk = acc + (size_t)kCoopMaxOwn * bs * nrhs;   // bs x bs, ld bs+1
  T* xb = dblk + (size_t)bs * ldd;                   // bs x nrhs
  const int G = gridDim.x, j = blockIdx.x, tid = threadIdx.x;
  const int nblk = (n + bs - 1) / bs;
  const int nown = (nblk - j + G - 1) / G;
  // non-transposed: L U x = P^T b (gather b[perm]); transposed: U^T L^T z = b, x = P z
  for (int o = 0; o < nown; ++o) {
    const int r0 = (j + o * G) * bs;
    for (int idx = tid; idx < bs * nrhs; idx += blockDim.x) {
      const int r = idx % bs, c = idx / bs;
      acc[(size_t)o * bs * nrhs + idx] =
          (r0 + r < n) ? Bin[(trans ? r0 + r : perm[r0 + r]) + (size_t)c * ldb] : T(0);
    }
  }
  for (int pass = 0; pass < 2; ++pass) {
    const bool lower = pass == 0;  // the first pass walks the blocks forward
    const T* Inv = (lower != (trans != 0)) ? Linv : Uinv;
    for (int step = 0; step < nblk; ++step) {
      const int b = lower ? step : nblk - 1 - step;
      const int k0 = b * bs, kb = min(bs, n - k0);
      if (b % G == j) {
        const int o = b / G;
        __syncthreads();
        if (!trans)
          stage_block(dblk, ldd, Inv + (size_t)b * bs * bs, bs, bs, bs);
        else
          stage_block_t(dblk, ldd, Inv + (size_t)b * bs * bs, bs, bs, bs);
        __syncthreads();
        for (int idx = tid; idx < kb * nrhs; idx += blockDim.x) {
          const int r = idx % kb, c = idx / kb;
          const T* a = acc + (size_t)o * bs * nrhs + (size_t)c * bs;
          T sum = T(0);
          for (int k = 0; k < kb; ++k) sum += dblk[r + k * ldd] * a[k];
          X[k0 + r + (size_t)c * ldx] = sum;
        }
      }
      grid.sync();
      __syncthreads();
      for (int idx = tid; idx < kb * nrhs; idx += blockDim.x) xb[idx] = X[k0 + idx % kb + (size_t)(idx / kb) * ldx];
      for (int o = 0; o < nown; ++o) {
        const int ob = j + o * G;
        if (lower ? ob <= b : ob >= b) continue;
        const int r0 = ob * bs;
        const int rb = min(bs, n - r0);
        __syncthreads();
        if (!trans)
          stage_block(dblk, ldd, LU + (size_t)k0 * lda + r0, lda, rb, kb);
        else  // op(A)[ob rows, b cols] = A[b rows, ob cols]^T
          stage_block_t(dblk, ldd, LU + (size_t)r0 * lda + k0, lda, rb, kb);
        __syncthreads();
        for (int idx = tid; idx < rb * nrhs; idx += blockDim.x) {
          const int r = idx % rb, c = idx / rb;
          T sum = T(0);
          for (int k = 0; k < kb; ++k) sum += dblk[r + k * ldd] * xb[k + c * kb];
          acc[(size_t)o * bs * nrhs + r + (size_t)c * bs] -= sum;
        }
      }
    }
    // second pass starts from the forward result held in X for the owned rows
    __syncthreads();
    for (int o = 0; o < nown; ++o) {
      const int r0 = (j + o * G) * bs;
      for (int idx = tid; idx < bs * nrhs; idx += blockDim.x) {
        const int r = idx % bs, c = idx / bs;
        acc[(size_t)o * bs * nrhs + idx] = (r0 + r < n) ? X[r0 + r + (size_t)c * ldx] : T(0);
      }
    }
    grid.sync();
  }
  if (trans) {
    // x = P z: acc holds z on the owned rows; row perm[i] of x is row i of z
    for (int o = 0; o < nown; ++o) {
      const int r0 = (j + o * G) * bs;
      for (int idx = tid; idx < bs * nrhs; idx += blockDim.x) {
        const int r = idx % bs, c = idx / bs;
        if (r0 + r < n) X[perm[r0 + r] + (size_t)c * ldx] = acc[(size_t)o * bs * nrhs + idx];
      }
    }
  }
}

// Cluster triangular solves with one large factored matrix: same contract as
// trsv_coop_kernel (X = A^{-1} B or A^{-T} B, nrhs <= kCoopMaxRhs, bs = 64
// inverted diagonal blocks), run by ONE thread-block cluster.  Row block b is
// owned by CTA b % CL, which keeps its right-hand-side accumulators in shared
// memory across both passes.  Per block step: the owner forms x_b = inv_b acc_b
// into a double-buffered shared array, one cluster barrier publishes it, every
// CTA reads it through distributed shared memory and subtracts op(A)[own, b] x_b
// from the blocks it owns.  A cluster barrier is a few hundred cycles, against
// microseconds for a grid-wide barrier.
constexpr int kClBs = 64;

// y[r][c] (+)= sum_k op(A)[r][k] x[k][c] for r < rb, k < kb, op(A)[r][k] =
// A[r + k*lda] (trans 0, rows contiguous) or A[k + r*lda] (trans 1).
// x: shared, ld kClBs, ZERO beyond row kb.  Non-transposed partials go to
// red[4][kClBs][nrhs] (summed by cl_reduce after a barrier); transposed
// results are written to y directly (scaled by sgn, accumulated when acc_mode).
// The column loop is a runtime loop and the FMA chain has no per-column
// predicate: GB300 retires about two FP64 FMAs per clock per SM, so issued but
// predicated-off FP64 instructions cost as much as useful ones.
// A tile (rb x kb, rows r, k columns from A with leading dimension lda) as held
// by one thread of cl_gemv_n: row tid % 64, the k-quarter tid / 64.
template <typename T>
__device__ __forceinline__ void cl_load_n(const T* __restrict__ A, int lda, int rb, int kb, T (&a)[kClBs / 4]) {
  const int tid = threadIdx.x;
  const int r = tid & (kClBs - 1), kq = tid >> 6;  // 256 threads: 64 rows x 4 k-quarters
  const int kbeg = kq * (kClBs / 4);
#pragma unroll
  for (int t = 0; t < kClBs / 4; ++t) a[t] = (r < rb && kbeg + t < kb) ? A[r + (size_t)(kbeg + t) * lda] : T(0);
}

// Partial products of a loaded tile with x (nrhs columns of ld kClBs) into red.
template <typename T>
__device__ __forceinline__ void cl_mul_n(const T (&a)[kClBs / 4], const T* x, int nrhs, T* red) {
  const int tid = threadIdx.x;
  const int r = tid & (kClBs - 1), kq = tid >> 6;
  const int kbeg = kq * (kClBs / 4);
  for (int c = 0; c < nrhs; ++c) {
    const T* xc = x + kbeg + c * kClBs;
    T part0 = T(0), part1 = T(0);
#pragma unroll
    for (int t = 0; t < kClBs / 4; t += 2) {
      part0 += a[t] * xc[t];
      part1 += a[t + 1] * xc[t + 1];
    }
    red[(kq * kClBs + r) + (size_t)c * 4 * kClBs] = part0 + part1;
  }
}

// y = A x for an rb x kb tile: partial sums of 64 rows x 4 k-quarters into red
// (cl_reduce finishes them).
template <typename T>
__device__ __forceinline__ void cl_gemv_n(const T* __restrict__ A, int lda, int rb, int kb, const T* x, int nrhs,
                                          T* red) {
  T a[kClBs / 4];
  cl_load_n(A, lda, rb, kb, a);
  cl_mul_n(a, x, nrhs, red);
}

template <typename T>
__device__ __forceinline__ T cl_reduce(const T* red, int r, int c) {
  const T* q = red + r + (size_t)c * 4 * kClBs;
  return (q[0] + q[kClBs]) + (q[2 * kClBs] + q[3 * kClBs]);
}

template <typename T>
__device__ __forceinline__ void cl_gemv_t(const T* __restrict__ A, int lda, int rb, int kb, const T* x, int nrhs,
                                          T* y, T sgn, bool acc_mode) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  for (int r = warp; r < rb; r += nw) {
    const T a0 = lane < kb ? A[lane + (size_t)r * lda] : T(0);
    const T a1 = lane + 32 < kb ? A[lane + 32 + (size_t)r * lda] : T(0);
    for (int c = 0; c < nrhs; ++c) {
      T v = a0 * x[lane + c * kClBs] + a1 * x[lane + 32 + c * kClBs];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) y[r + c * kClBs] = acc_mode ? y[r + c * kClBs] + sgn * v : sgn * v;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256) trsv_cluster_kernel(const T* __restrict__ LU, int lda, int n,
                                                           const int* __restrict__ perm, const T* __restrict__ Linv,
                                                           const T* __restrict__ Uinv, const T* __restrict__ Bin,
                                                           int ldb, T* X, int ldx, int nrhs, int trans, int own_max) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int bs = kClBs;
  const int CL = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int tid = threadIdx.x;
  const int vb = bs * kCoopMaxRhs;                 // one block of right-hand sides (ld bs)
  T* acc = reinterpret_cast<T*>(smem_raw);         // own_max x vb
  T* xbuf = acc + (size_t)own_max * vb;            // 2 x vb (published x_b)
  T* xloc = xbuf + 2 * (size_t)vb;                 // vb (local copy of the current x_b)
  T* red = xloc + vb;                              // own_max x 4 x vb
  const int nblk = (n + bs - 1) / bs;
  const int nown = rank < nblk ? (nblk - 1 - rank) / CL + 1 : 0;
  for (int o = 0; o < nown; ++o) {
    const int r0 = (rank + o * CL) * bs;
    for (int idx = tid; idx < bs * nrhs; idx += blockDim.x) {
      const int r = idx % bs, c = idx / bs;
      acc[(size_t)o * vb + idx] = (r0 + r < n) ? Bin[(trans ? r0 + r : perm[r0 + r]) + (size_t)c * ldb] : T(0);
    }
  }
  // Non-transposed solves load their tiles one step ahead: at the start of a
  // step, the tiles of this step's updates (which do not depend on x_b) and the
  // next step's owner its inverted diagonal block, so the loads overlap the
  // owner's product and the cluster barrier.  Blocks past the second owned one
  // load at use.
  constexpr int kPre = 2;
  T pre[kPre][kClBs / 4];
  T ipre[kClBs / 4];
  int ipre_step = -1;  // step_all whose inverse tile ipre holds
  auto step_block = [&](int sa) { return sa < nblk ? sa : 2 * nblk - 1 - sa; };  // b of a step_all
  auto step_inv = [&](int sa) { return (sa < nblk) != (trans != 0) ? Linv : Uinv; };
  if (!trans && rank == step_block(0) % CL) {
    const int b = step_block(0), kb = min(bs, n - b * bs);
    cl_load_n(step_inv(0) + (size_t)b * bs * bs, bs, kb, kb, ipre);
    ipre_step = 0;
  }
  int step_all = 0;
  for (int pass = 0; pass < 2; ++pass) {
    const bool fwd = pass == 0;
    const T* Inv = (fwd != (trans != 0)) ? Linv : Uinv;
    for (int step = 0; step < nblk; ++step, ++step_all) {
      const int b = fwd ? step : nblk - 1 - step;
      const int k0 = b * bs, kb = min(bs, n - k0);
      const int owner = b % CL;
      T* xb = xbuf + (size_t)(step_all & 1) * vb;
      T ib_now[kClBs / 4];
      bool ib_ready = false;
      if (!trans) {
        if (ipre_step == step_all) {
#pragma unroll
          for (int t = 0; t < kClBs / 4; ++t) ib_now[t] = ipre[t];
          ib_ready = true;
        }
#pragma unroll
        for (int o = 0; o < kPre; ++o) {
          const int ob = rank + o * CL;
          if (o < nown && (fwd ? ob > b : ob < b))
            cl_load_n(LU + (size_t)k0 * lda + ob * bs, lda, min(bs, n - ob * bs), kb, pre[o]);
        }
        const int sn = step_all + 1;
        if (sn < 2 * nblk && rank == step_block(sn) % CL) {
          const int bn = step_block(sn), kbn = min(bs, n - bn * bs);
          cl_load_n(step_inv(sn) + (size_t)bn * bs * bs, bs, kbn, kbn, ipre);
          ipre_step = sn;
        }
      }
      if (rank == owner) {
        const int o = b / CL;
        T* a = acc + (size_t)o * vb;
        const T* Ib = Inv + (size_t)b * bs * bs;
        __syncthreads();
        if (!trans) {
          if (ib_ready)
            cl_mul_n(ib_now, a, nrhs, red);
          else
            cl_gemv_n(Ib, bs, kb, kb, a, nrhs, red);
          __syncthreads();
          for (int idx = tid; idx < kb * nrhs; idx += blockDim.x) {
            const int r = idx % kb, c = idx / kb;
            xb[r + c * bs] = cl_reduce(red, r, c);
          }
        } else {
          cl_gemv_t(Ib, bs, kb, kb, a, nrhs, xb, T(1), false);
        }
        __syncthreads();
        // keep x_b: the next pass starts from it; the last pass is the output
        for (int idx = tid; idx < kb * nrhs; idx += blockDim.x) {
          const int r = idx % kb, c = idx / kb;
          const T v = xb[r + c * bs];
          if (fwd)
            a[r + c * bs] = v;
          else if (!trans)
            X[k0 + r + (size_t)c * ldx] = v;
          else
            X[perm[k0 + r] + (size_t)c * ldx] = v;
        }
      }
      cluster.sync();
      const T* src = cluster.map_shared_rank(xb, owner);
      for (int idx = tid; idx < bs * nrhs; idx += blockDim.x) {
        const int r = idx % bs, c = idx / bs;
        xloc[r + c * bs] = r < kb ? src[r + c * bs] : T(0);
      }
      __syncthreads();
      // blocks still to come in this pass: b+1.. (forward) or ..b-1 (backward)
      int nupd = 0;
      // the prefetched tiles (static indices keep them in registers), then the rest
#pragma unroll
      for (int o = 0; o < kPre; ++o) {
        const int ob = rank + o * CL;
        if (trans || o >= nown || (fwd ? ob <= b : ob >= b)) continue;
        cl_mul_n(pre[o], xloc, nrhs, red + (size_t)o * 4 * vb);
        ++nupd;
      }
      for (int o = trans ? 0 : kPre; o < nown; ++o) {
        const int ob = rank + o * CL;
        if (fwd ? ob <= b : ob >= b) continue;
        const int r0 = ob * bs, rb = min(bs, n - r0);
        if (!trans)
          cl_gemv_n(LU + (size_t)k0 * lda + r0, lda, rb, kb, xloc, nrhs, red + (size_t)o * 4 * vb);
        else
          cl_gemv_t(LU + (size_t)r0 * lda + k0, lda, rb, kb, xloc, nrhs, acc + (size_t)o * vb, T(-1), true);
        ++nupd;
      }
      if (!trans && nupd > 0) {
        __syncthreads();
        for (int o = 0; o < nown; ++o) {
          const int ob = rank + o * CL;
          if (fwd ? ob <= b : ob >= b) continue;
          const int rb = min(bs, n - ob * bs);
          for (int idx = tid; idx < rb * nrhs; idx += blockDim.x) {
            const int r = idx % rb, c = idx / rb;
            acc[(size_t)o * vb + r + c * bs] -= cl_reduce(red + (size_t)o * 4 * vb, r, c);
          }
        }
      }
    }
  }
  cluster.sync();  // no CTA leaves while its shared memory may still be read
}

// Split-K narrow GEMM for one tall matrix: C += alpha * A[:, kchunk] B[kchunk, :]
// accumulated with atomics (C already scaled by beta).  grid (ceil(m/256), nsplit).
template <typename T, int NC>
__global__ void __launch_bounds__(256) gemm_narrow_splitk_kernel(int m, int n, int k, int kchunk, T alpha,
                                                                const T* __restrict__ A, int lda,
                                                                const T* __restrict__ B, int ldb, T* C, int ldc) {
  __shared__ T Bs[NC * 256];
  const int k0 = blockIdx.y * kchunk;
  const int kc = min(kchunk, k - k0);
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  for (int idx = threadIdx.x; idx < 256 * NC; idx += blockDim.x) {
    const int kk = idx % 256, c = idx / 256;
    Bs[c * 256 + kk] = (kk < kc && c < n) ? B[(k0 + kk) + (size_t)c * ldb] : T(0);
  }
  __syncthreads();
  if (r >= m || kc <= 0) return;
  T acc[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) acc[c] = T(0);
  const T* ap = A + r + (size_t)k0 * lda;
  for (int kk = 0; kk < kc; ++kk) {
    const T a = ap[(size_t)kk * lda];
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[c] += a * Bs[c * 256 + kk];
  }
#pragma unroll
  for (int c = 0; c < NC; ++c)
    if (c < n) atomicAdd(C + r + (size_t)c * ldc, alpha * acc[c]);
}

// Narrow transposed GEMM: C (m x n, n <= NC) = beta C + alpha A^T B with A k x m.
// One warp per row of C: the lanes read the column of A and of B (coalesced)
// and reduce with shuffles.  grid (ceil(m/8), 1, batch), 256 threads.
template <typename T, int NC>
__global__ void __launch_bounds__(256) gemm_tn_narrow_kernel(int m, int n, int k, T alpha, const T* __restrict__ A,
                                                            const long long* offA, long long strideA, int lda,
                                                            const T* __restrict__ B, const long long* offB,
                                                            long long strideB, int ldb, T beta, T* C,
                                                            const long long* offC, long long strideC, int ldc) {
  const int bz = blockIdx.z;
  A += batch_off(offA, strideA, bz);
  B += batch_off(offB, strideB, bz);
  C += batch_off(offC, strideC, bz);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * 8 + warp;
  if (r >= m) return;
  const T* ac = A + (size_t)r * lda;
  T acc[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) acc[c] = T(0);
  for (int kk = lane; kk < k; kk += 32) {
    const T a = ac[kk];
#pragma unroll
    for (int c = 0; c < NC; ++c)
      if (c < n) acc[c] += a * B[kk + (size_t)c * ldb];
  }
#pragma unroll
  for (int c = 0; c < NC; ++c) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
  }
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      if (c >= n) break;
      T* cp = C + r + (size_t)c * ldc;
      *cp = (beta == T(0) ? T(0) : beta * *cp) + alpha * acc[c];
    }
  }
}

template <typename T>
__global__ void scale_kernel(T* C, int m, int n, int ldc, T beta) {
  const long long tot = (long long)m * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    T* cp = C + (i % m) + (size_t)(i / m) * ldc;
    *cp = beta == T(0) ? T(0) : beta * *cp;
  }
}

// ---------------------------------------------------------------------------
// Large single-matrix LU (FP64 interface blocks): host loop over panels.

// Panel factorization in global memory: rows [k0, n), columns [k0, k0+nb).
template <typename T>
__global__ void __launch_bounds__(1024) biglu_panel_kernel(T* A, int lda, int n, int k0, int nb, int* ipiv,
                                                          int* info) {
  __shared__ T sv[33];
  __shared__ int si[33];
  const int tid = threadIdx.x;
  for (int j = 0; j < nb; ++j) {
    const int col = k0 + j;
    T* cj = A + (size_t)col * lda;
    mag_t<T> best = 0;
    int bi = INT_MAX;
    for (int r = col + tid; r < n; r += blockDim.x) {
      const mag_t<T> a = mag_key(cj[r]);
      if (bi == INT_MAX || a > best) {
        best = a;
        bi = r;
      }
    }
    int pr = cta_argmax<T>(best, bi, sv, si);
    if (pr == INT_MAX) pr = col;
    if (tid == 0) ipiv[col] = pr;
    if (pr != col) {
      for (int c = tid; c < nb; c += blockDim.x) {
        T* cc = A + (size_t)(k0 + c) * lda;
        T t = cc[col];
        cc[col] = cc[pr];
        cc[pr] = t;
      }
    }
    __syncthreads();
    const T d = cj[col];
    if (d == T(0) || d != d) {
      if (tid == 0 && info && *info == 0) *info = col + 1;
    } else {
      const T rd = cta_recip(d, sv + 32);
      for (int r = col + 1 + tid; r < n; r += blockDim.x) {
        const T l = cj[r] * rd;
        cj[r] = l;
        for (int c = j + 1; c < nb; ++c) {
          T* cc = A + (size_t)(k0 + c) * lda;
          cc[r] -= l * cc[col];
        }
      }
    }
    __syncthreads();
  }
}

// Panel factorization held in the distributed shared memory of one thread-block
// cluster of CL CTAs: CTA r keeps physical panel rows [r*R, (r+1)*R) of the
// m x nb panel (rows k0.. of columns k0..k0+nb), one row per thread (R <= 256).
// Rows never move: each thread keeps the logical index of its row in a
// register.  One column j costs one cluster barrier, split into arrive and wait:
//   1. every CTA finds its best candidate (largest magnitude, smallest logical
//      index on ties) among its rows with logical index >= j and pushes it --
//      key, logical index, physical row and the row's nb values -- into a
//      mailbox slot of every CTA of the cluster (DSMEM stores);
//   2. arrive; while the barrier completes, each thread applies the previous
//      pivot's update to columns j+1.. of its row (the update is deferred by
//      one column: only column j has to be current for the search);
//   3. wait; every warp reduces the CL candidates from its own CTA's mailbox,
//      so the pivot row is read from local shared memory; each thread relabels
//      its row for the interchange, forms its multiplier and updates column j+1.
// The pushed candidate row already includes the deferred update, computed by
// the pusher from the owner's multiplier.  Mailboxes are triple-buffered: a
// CTA pushes column j+1 only after the barrier of column j, which every thread
// reaches only after the deferred update that still reads the pivot row of
// column j-1.  The pivot sequence is LAPACK's.  At the end each thread writes
// its row to its logical position, and CTA 0 gathers the unit-lower nb x nb
// triangle (pushed by the owners) and writes its inverse to linv.
// Shared memory: see panel_cluster_smem_bytes.  grid = CL (one cluster).
__host__ __device__ inline size_t panel_cluster_smem_bytes(int m, int nb, int R, size_t elem) {
  (void)m;
  constexpr int kCLMax = 16;
  return ((size_t)R * nb + R + 3 * (size_t)kCLMax * nb + 2 * (size_t)nb * (nb + 1)) * elem +
         3 * (size_t)kCLMax * (elem + 2 * sizeof(int));
}

__device__ __forceinline__ void cluster_arrive_release() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_wait_acquire() {
  asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// (key, logical index, slot) candidate merge with the LAPACK tie-break.
template <typename K>
__device__ __forceinline__ void argmax_merge3(K& v, int& i, int& sl, K v2, int i2, int s2) {
  if (v2 > v || (v2 == v && i2 < i)) {
    v = v2;
    i = i2;
    sl = s2;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) biglu_panel_cluster_kernel(T* A, int lda, int n, int k0, int nb, int R,
                                                                  int* ipiv, int* info, T* linv) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  using K = mag_t<T>;
  constexpr int kCLMax = 16;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int m = n - k0;
  const int ldx = nb + 1;
  T* P = reinterpret_cast<T*>(smem_raw);    // R x nb, ld R (physical rows)
  T* lcol = P + (size_t)R * nb;              // R: each row's multiplier of the previous column
  T* mrow = lcol + R;                        // [3][kCLMax][nb] pushed candidate rows
  T* Ls = mrow + 3 * kCLMax * nb;            // nb x nb, ld nb+1: gathered L11 (CTA 0)
  T* Xs = Ls + (size_t)nb * ldx;             // nb x nb, ld nb+1: its inverse
  K* mkey = reinterpret_cast<K*>(Xs + (size_t)nb * ldx);  // [3][kCLMax]
  int* mli = reinterpret_cast<int*>(mkey + 3 * kCLMax);    // [3][kCLMax] logical index
  int* mph = mli + 3 * kCLMax;                              // [3][kCLMax] physical row
  __shared__ K wk[8];
  __shared__ int wi[8];
  __shared__ int ws[8];
  const int CL = (int)cluster.num_blocks();
  const int rk = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int g0 = rk * R;
  const int rows = max(0, min(R, m - g0));
  const bool own = tid < rows;
  for (int c = 0; c < nb; ++c)
    for (int i = tid; i < rows; i += blockDim.x) cp_async_elem(&P[i + (size_t)c * R], &A[(size_t)(k0 + c) * lda + k0 + g0 + i]);
  cp_async_wait_all();
  int my_li = own ? g0 + tid : INT_MAX;
  T l_prev = T(0);              // this row's multiplier of the previous pivot (0: none)
  const T* prow_prev = nullptr;  // previous pivot row (mailbox)
  cluster.sync();  // every CTA of the cluster runs before the first DSMEM store
  for (int j = 0; j < nb && j < m; ++j) {
    const int buf = j % 3;
    // (a) local candidate among this thread's row, then the warp's and the CTA's
    K best = 0;
    int bi = INT_MAX, bs = -1;
    if (own && my_li >= j) {
      best = mag_key(P[tid + (size_t)j * R]);
      bi = my_li;
      bs = tid;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const K v2 = __shfl_xor_sync(0xffffffffu, best, o);
      const int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
      const int s2 = __shfl_xor_sync(0xffffffffu, bs, o);
      argmax_merge3(best, bi, bs, v2, i2, s2);
    }
    if (lane == 0) {
      wk[warp] = best;
      wi[warp] = bi;
      ws[warp] = bs;
    }
    if (own) lcol[tid] = l_prev;
    __syncthreads();  // (1) warp candidates and multipliers
    if (warp == 0) {
      K v = lane < nwarps ? wk[lane] : K(0);
      int i = lane < nwarps ? wi[lane] : INT_MAX;
      int sl = lane < nwarps ? ws[lane] : -1;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const K v2 = __shfl_xor_sync(0xffffffffu, v, o);
        const int i2 = __shfl_xor_sync(0xffffffffu, i, o);
        const int s2 = __shfl_xor_sync(0xffffffffu, sl, o);
        argmax_merge3(v, i, sl, v2, i2, s2);
      }
      // push the candidate to slot rk of every CTA's mailbox
      if (i != INT_MAX && lane < nb) {
        T x = P[sl + (size_t)lane * R];
        if (prow_prev && lane > j) x -= lcol[sl] * prow_prev[lane];
        for (int q = 0; q < CL; ++q) *cluster.map_shared_rank(&mrow[(buf * kCLMax + rk) * nb + lane], q) = x;
      }
      if (lane < CL) {
        *cluster.map_shared_rank(&mkey[buf * kCLMax + rk], lane) = v;
        *cluster.map_shared_rank(&mli[buf * kCLMax + rk], lane) = i;
        *cluster.map_shared_rank(&mph[buf * kCLMax + rk], lane) = i == INT_MAX ? -1 : g0 + sl;
      }
    }
    __syncthreads();  // (2) the candidate row is read before its owner updates it below
    cluster_arrive_release();
    // (b) deferred update of the previous pivot on columns j+1.. of this row
    if (own && l_prev != T(0))
      for (int c = j + 1; c < nb; ++c) P[tid + (size_t)c * R] -= l_prev * prow_prev[c];
    cluster_wait_acquire();
    // (c) every warp reduces the CL candidates of its own mailbox
    K v = lane < CL ? mkey[buf * kCLMax + lane] : K(0);
    int wli = lane < CL ? mli[buf * kCLMax + lane] : INT_MAX;
    int wq = lane;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const K v2 = __shfl_xor_sync(0xffffffffu, v, o);
      const int i2 = __shfl_xor_sync(0xffffffffu, wli, o);
      const int s2 = __shfl_xor_sync(0xffffffffu, wq, o);
      argmax_merge3(v, wli, wq, v2, i2, s2);
    }
    const int piv = wli == INT_MAX ? j : wli;
    const T* prow = &mrow[(buf * kCLMax + (wli == INT_MAX ? 0 : wq)) * nb];
    const int php = wli == INT_MAX ? -1 : mph[buf * kCLMax + wq];
    if (rk == 0 && tid == 0) ipiv[k0 + j] = k0 + piv;
    const bool ok = wli != INT_MAX && mag_key(prow[j]) != 0;  // zero or NaN pivot: integer test
    if (!ok && rk == 0 && tid == 0 && info && *info == 0) *info = k0 + j + 1;
    T rd = T(0);
    if (ok) {
      if (lane == 0) rd = recip_newton(prow[j]);
      rd = __shfl_sync(0xffffffffu, rd, 0);
    }
    // (d) interchange (labels only), multiplier, update of column j+1
    l_prev = T(0);
    if (own) {
      if (g0 + tid == php)
        my_li = j;
      else if (my_li == j)
        my_li = piv;
      if (ok && my_li > j) {
        const T l = P[tid + (size_t)j * R] * rd;
        P[tid + (size_t)j * R] = l;
        if (j + 1 < nb) P[tid + (size_t)(j + 1) * R] -= l * prow[j + 1];
        l_prev = l;
      }
    }
    prow_prev = prow;
  }
  // every update of this thread's row is its own: write it back
  if (own)
    for (int c = 0; c < nb; ++c) A[(size_t)(k0 + c) * lda + k0 + my_li] = P[tid + (size_t)c * R];
  if (linv && nb <= m) {
    // owners of logical rows 0..nb-1 push their first nb values to CTA 0
    if (own && my_li < nb)
      for (int c = 0; c < nb; ++c) *cluster.map_shared_rank(&Ls[my_li + (size_t)c * ldx], 0) = P[tid + (size_t)c * R];
    cluster.sync();
    if (rk == 0) {
      // L11^{-1} by forward substitution, one warp per group of columns and one
      // lane per row (nb <= 32): step k broadcasts x[k] and updates rows i > k,
      // so the dependent chain is nb steps long for all the warp's columns at once.
      constexpr int kCols = 4;
      for (int c0 = warp * kCols; c0 < nb; c0 += nwarps * kCols) {
        T x[kCols];
#pragma unroll
        for (int q = 0; q < kCols; ++q) x[q] = lane == c0 + q ? T(1) : T(0);
        for (int k = c0; k < nb - 1; ++k) {
          const T lik = lane > k && lane < nb ? Ls[lane + (size_t)k * ldx] : T(0);
#pragma unroll
          for (int q = 0; q < kCols; ++q) {
            const T xk = __shfl_sync(0xffffffffu, x[q], k);
            x[q] -= lik * xk;
          }
        }
#pragma unroll
        for (int q = 0; q < kCols; ++q)
          if (c0 + q < nb && lane < nb) Xs[lane + (size_t)(c0 + q) * ldx] = x[q];
      }
      __syncthreads();
      for (int idx = tid; idx < nb * nb; idx += blockDim.x) linv[idx] = Xs[(idx % nb) + (idx / nb) * ldx];
    }
  }
}

// Inverse of the nb x nb diagonal triangle A[k0:k0+nb, k0:k0+nb] (unit lower if
// upper == 0, upper otherwise), one CTA per block; blocks k0 = blk * bs.
// out: nblk blocks of bs x bs (column-major, ld bs), zero outside the triangle.
template <typename T>
__global__ void __launch_bounds__(128) tri_inv_blocks_kernel(const T* A, int lda, int n, int bs, int upper, T* out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ld = bs + 1;
  T* D = reinterpret_cast<T*>(smem_raw);  // bs x bs, ld bs+1
  T* Xs = D + (size_t)bs * ld;              // bs x bs, ld bs+1 (column c = thread c)
  const int blk = blockIdx.x;
  const int k0 = blk * bs, nb = min(bs, n - k0);
  T* O = out + (size_t)blk * bs * bs;
  T* rdiag = Xs + (size_t)bs * ld;           // bs: reciprocals of the diagonal (upper)
  // eight loads in flight per thread before their stores
  for (int base = threadIdx.x; base < bs * bs; base += 8 * blockDim.x) {
    T t[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = base + u * blockDim.x;
      const int i = idx % bs, c = idx / bs;
      t[u] = (idx < bs * bs && i < nb && c < nb) ? A[(size_t)(k0 + c) * lda + k0 + i] : T(0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = base + u * blockDim.x;
      if (idx < bs * bs) {
        const int i = idx % bs, c = idx / bs;
        D[i + c * ld] = t[u];
        Xs[i + c * ld] = T(0);
      }
    }
  }
  __syncthreads();
  if (upper)
    for (int i = threadIdx.x; i < nb; i += blockDim.x) rdiag[i] = T(1) / D[i + i * ld];
  __syncthreads();
  // one thread per column; each dot product is split over four partial sums,
  // which cuts the dependent chain of the substitution (FP64 latency) by four
  for (int c = threadIdx.x; c < nb; c += blockDim.x) {
    T* x = Xs + c * ld;
    if (!upper) {
      x[c] = T(1);
      for (int i = c + 1; i < nb; ++i) {
        T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
        int k = c;
        for (; k + 3 < i; k += 4) {
          s0 -= D[i + k * ld] * x[k];
          s1 -= D[i + (k + 1) * ld] * x[k + 1];
          s2 -= D[i + (k + 2) * ld] * x[k + 2];
          s3 -= D[i + (k + 3) * ld] * x[k + 3];
        }
        for (; k < i; ++k) s0 -= D[i + k * ld] * x[k];
        x[i] = (s0 + s1) + (s2 + s3);
      }
    } else {
      x[c] = rdiag[c];
      for (int i = c - 1; i >= 0; --i) {
        T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
        int k = i + 1;
        for (; k + 3 <= c; k += 4) {
          s0 -= D[i + k * ld] * x[k];
          s1 -= D[i + (k + 1) * ld] * x[k + 1];
          s2 -= D[i + (k + 2) * ld] * x[k + 2];
          s3 -= D[i + (k + 3) * ld] * x[k + 3];
        }
        for (; k <= c; ++k) s0 -= D[i + k * ld] * x[k];
        x[i] = ((s0 + s1) + (s2 + s3)) * rdiag[i];
      }
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < bs * bs; idx += blockDim.x) {
    const int i = idx % bs, c = idx / bs;
    O[idx] = Xs[i + c * ld];
  }
}

// X[k0:k0+nb, :] = Inv * X[k0:k0+nb, :] with a precomputed nb x nb inverse
// (ld bs); grid: column tiles of kTrsmCols (narrow tiles spread the FP64 work
// over every SM).
constexpr int kTrsmCols = 8;
template <typename T>
__global__ void __launch_bounds__(256) trsm_inv_kernel(const T* Inv, int bs, int k0, int nb, T* X, int ldx,
                                                      int ncols) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* Is = reinterpret_cast<T*>(smem_raw);  // bs x bs
  T* Xs = Is + bs * bs;                    // bs x kTrsmCols
  const int c0 = blockIdx.x * kTrsmCols;
  const int nc = min(kTrsmCols, ncols - c0);
  // eight loads in flight per thread before their stores (one memory latency per
  // eight elements instead of one per element)
  for (int base = threadIdx.x; base < bs * bs; base += 8 * blockDim.x) {
    T t[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = base + u * blockDim.x;
      t[u] = idx < bs * bs ? Inv[idx] : T(0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = base + u * blockDim.x;
      if (idx < bs * bs) Is[idx] = t[u];
    }
  }
  for (int idx = threadIdx.x; idx < nb * nc; idx += blockDim.x) {
    const int i = idx % nb, c = idx / nb;
    Xs[i + c * bs] = X[(size_t)(c0 + c) * ldx + k0 + i];
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < nb * nc; idx += blockDim.x) {
    const int i = idx % nb, c = idx / nb;
    // one running sum in ascending k: at N = 4.4M four interleaved partial sums
    // here cost the FP32 interface two more refinement steps to 1e-10 (12 vs 10)
    T s = T(0);
    for (int k = 0; k < nb; ++k) s += Is[i + k * bs] * Xs[k + c * bs];
    X[(size_t)(c0 + c) * ldx + k0 + i] = s;
  }
}

// Apply the panel's row interchanges ipiv[k0 .. k0+nb) to every column outside
// the panel (one thread per column).
template <typename T>
__global__ void biglu_swap_kernel(T* A, int lda, int ncols_total, int k0, int nb, const int* ipiv) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncols_total - nb) return;
  const int col = c < k0 ? c : c + nb;
  T* cp = A + (size_t)col * lda;
  for (int j = 0; j < nb; ++j) {
    const int pr = ipiv[k0 + j];
    if (pr != k0 + j) {
      T t = cp[k0 + j];
      cp[k0 + j] = cp[pr];
      cp[pr] = t;
    }
  }
}

// Row interchanges ipiv[k0 .. k0+nb) of one panel applied to the columns
// [c_lo, k0) and [k0+nb, c_hi) (one thread per column).
template <typename T>
__global__ void swap_cols_kernel(T* A, int lda, int c_lo, int c_hi, int k0, int nb, const int* ipiv) {
  const int c = c_lo + blockIdx.x * blockDim.x + threadIdx.x;
  const int col = c < k0 ? c : c + nb;
  if (col >= c_hi) return;
  T* cp = A + (size_t)col * lda;
  for (int j = 0; j < nb; ++j) {
    const int pr = ipiv[k0 + j];
    if (pr != k0 + j) {
      T t = cp[k0 + j];
      cp[k0 + j] = cp[pr];
      cp[pr] = t;
    }
  }
}

// A panel's row interchanges given as a gather list (gath[0] = count <= 2 kNB,
// then (destination, source) row pairs) applied to the columns [c_lo, k0) and
// [k0+nb, c_hi): every moved value of a column is loaded before any is stored,
// so the loads of a column are all in flight at once.
template <typename T>
__global__ void __launch_bounds__(128) swap_gather_kernel(T* A, int lda, int c_lo, int c_hi, int k0, int nb,
                                                          const int* __restrict__ gath) {
  __shared__ int g[1 + 4 * kNB];
  for (int i = threadIdx.x; i < 1 + 4 * kNB; i += blockDim.x) g[i] = gath[i];
  __syncthreads();
  const int c = c_lo + blockIdx.x * blockDim.x + threadIdx.x;
  const int col = c < k0 ? c : c + nb;
  if (col >= c_hi) return;
  T* cp = A + (size_t)col * lda;
  const int cnt = g[0];
  T v[2 * kNB];
#pragma unroll
  for (int t = 0; t < 2 * kNB; ++t)
    if (t < cnt) v[t] = cp[g[2 + 2 * t]];
#pragma unroll
  for (int t = 0; t < 2 * kNB; ++t)
    if (t < cnt) cp[g[1 + 2 * t]] = v[t];
}

// Net effect of the interchanges ipiv[k0 .. k0+npiv) (LAPACK order, rows of an
// n-row matrix) as a gather: out[0] = count, then count (destination, source)
// row pairs at out[1 + 2t], out[2 + 2t] (count <= 2 npiv).  One CTA; dynamic
// shared memory (n - k0) ints.
__global__ void rowperm_build_kernel(const int* ipiv, int k0, int npiv, int n, int* out);

// Applies a gather from rowperm_build_kernel to the columns [lo1, hi1) and
// [lo2, hi2) of A: every value of a column is read before any is written.
// kRowpermCols columns per CTA.
constexpr int kRowpermCols = 8;
constexpr int kRowpermMax = 2 * 256;
template <typename T>
__global__ void __launch_bounds__(256) rowperm_apply_kernel(T* A, int lda, int lo1, int hi1, int lo2, int hi2,
                                                            const int* perm) {
  __shared__ T vals[kRowpermMax * kRowpermCols];
  const int cnt = min(perm[0], kRowpermMax);
  const int n1 = max(0, hi1 - lo1);
  const int ncols = n1 + max(0, hi2 - lo2);
  const int cbase = blockIdx.x * kRowpermCols;
  const int nc = min(kRowpermCols, ncols - cbase);
  if (nc <= 0) return;
  for (int idx = threadIdx.x; idx < cnt * nc; idx += blockDim.x) {
    const int t = idx % cnt, ci = cbase + idx / cnt;
    const int col = ci < n1 ? lo1 + ci : lo2 + (ci - n1);
    vals[idx] = A[(size_t)col * lda + perm[2 + 2 * t]];
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < cnt * nc; idx += blockDim.x) {
    const int t = idx % cnt, ci = cbase + idx / cnt;
    const int col = ci < n1 ? lo1 + ci : lo2 + (ci - n1);
    A[(size_t)col * lda + perm[1 + 2 * t]] = vals[idx];
  }
}

// Triangular solve with the nb x nb diagonal block D = A[k0 : k0+nb, k0 : k0+nb]
// applied to rows [k0, k0+nb) of X (columns [0, ncols)):
//   upper == 0: X_blk = L_D^{-1} X_blk (unit lower);  upper == 1: X_blk = U_D^{-1} X_blk.
// grid: column tiles of 64.
template <typename T>
__global__ void __launch_bounds__(256) trsm_block_kernel(const T* A, int lda, int k0, int nb, T* X, int ldx,
                                                        int ncols, int upper) {
  __shared__ T Dsm[kNB * (kNB + 1)];
  __shared__ T Xs[kNB * 65];
  const int c0 = blockIdx.x * 64;
  const int nc = min(64, ncols - c0);
  const int tid = threadIdx.x;
  for (int idx = tid; idx < nb * nb; idx += blockDim.x) {
    const int r = idx % nb, c = idx / nb;
    Dsm[r + c * (kNB + 1)] = A[(size_t)(k0 + c) * lda + k0 + r];
  }
  for (int idx = tid; idx < nb * nc; idx += blockDim.x) {
    const int r = idx % nb, c = idx / nb;
    Xs[c + r * 65] = X[(size_t)(c0 + c) * ldx + k0 + r];
  }
  __syncthreads();
  if (tid < nc) {
    const int c = tid;
    if (!upper) {
      for (int i = 1; i < nb; ++i) {
        T s = Xs[c + i * 65];
        for (int k = 0; k < i; ++k) s -= Dsm[i + k * (kNB + 1)] * Xs[c + k * 65];
        Xs[c + i * 65] = s;
      }
    } else {
      for (int i = nb - 1; i >= 0; --i) {
        T s = Xs[c + i * 65];
        for (int k = i + 1; k < nb; ++k) s -= Dsm[i + k * (kNB + 1)] * Xs[c + k * 65];
        Xs[c + i * 65] = s / Dsm[i + i * (kNB + 1)];
      }
    }
  }
  __syncthreads();
  for (int idx = tid; idx < nb * nc; idx += blockDim.x) {
    const int r = idx % nb, c = idx / nb;
    X[(size_t)(c0 + c) * ldx + k0 + r] = Xs[c + r * 65];
  }
}

// Final row permutation of a sequence of interchanges: perm[i] = source row of row i.
__global__ void perm_from_ipiv_kernel(const int* ipiv, int n, int* perm);

// out[i, c] = in[perm[i], c]
template <typename T>
__global__ void permute_rows_kernel(const T* in, int ldi, T* out, int ldo, int n, int ncols, const int* perm) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)n * ncols) return;
  const int r = (int)(idx % n), c = (int)(idx / n);
  out[r + (size_t)c * ldo] = in[perm[r] + (size_t)c * ldi];
}

// ---------------------------------------------------------------------------
// Host-side launchers (defined in dense.cu for float and double).
template <typename T>
int gemm(cudaStream_t s, int m, int n, int k, T alpha, const T* A, const long long* offA, long long strideA,
         int lda, const T* B, const long long* offB, long long strideB, int ldb, T beta, T* C,
         const long long* offC, long long strideC, int ldc, int batch);

template <typename T>
int getrf_batched(cudaStream_t s, int n, int nc, T* A, const long long* offA, long long strideA, int lda,
                  int* piv, const long long* offP, long long strideP, int* info, int batch);

template <typename T>
int getrs_batched(cudaStream_t s, int n, int nrhs, const T* LU, const long long* offLU, long long strideLU,
                  int lda, const int* piv, const long long* offP, long long strideP, T* B,
                  const long long* offB, long long strideB, int ldb, int batch, bool lower = true,
                  bool upper = true);

// Tile policy of the FP32 products (gemm) issued by the calling host thread:
// 0 = 128 x 128 tiles where their grid fills the GPU, 64 x 64 otherwise; 1 =
// always 64 x 64.
void set_gemm_tiles(int policy);

// Large single-matrix LU in place (n x n, lda); ipiv/info device pointers.
// work: kNB*kNB elements (inverse of the current panel's unit-lower triangle).
// panel_kind 0: FP32 panels of up to 1536 rows in one CTA; 1: always
// the cluster panel kernel (same pivots and factors).
template <typename T>
int biglu(cudaStream_t s, T* A, int lda, int n, int* ipiv, int* info, T* work = nullptr, int panel_kind = 0);

// biglu in outer blocks of 256 columns: 32-column pivoted panels (panel_kind as
// for biglu) with their updates inside the outer block, then the update of the
// columns beyond it through inverted 64 x 64 triangles of its L11 and one
// product.  With side/fork/join/perm (perm: 1 + 2 * kRowpermMax ints), the
// update of the columns beyond the next outer block runs on the side stream
// while that block's panels are factored; the panels' interchanges reach the
// other columns as one gather after the block.  The elimination of biglu with
// the products grouped differently: the factors agree to rounding (and so do
// the pivots, but for near ties).  panel_linv: kNB x kNB elements; blk_linv:
// 256 x 64 elements.
// gath (1 + 4 kNB ints, may be null): one-CTA panels leave their interchanges
// there as a gather list, applied to the other columns in one pass of loads.
template <typename T>
int biglu_blocked(cudaStream_t s, T* A, int lda, int n, int* ipiv, int* info, T* panel_linv, T* blk_linv,
                  int panel_kind, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join, int* perm, int* gath);

// Inverses of the bs x bs diagonal triangles of a factored matrix:
// Linv/Uinv hold ceil(n/bs) blocks of bs x bs each.
template <typename T>
int tri_inv_blocks(cudaStream_t s, const T* LU, int lda, int n, int bs, T* Linv, T* Uinv);

// bigtrs with precomputed diagonal-block inverses (block size bs).
template <typename T>
int bigtrs_inv(cudaStream_t s, const T* LU, int lda, int n, const int* perm, const T* Linv, const T* Uinv, int bs,
               const T* B, int ldb, T* X, int ldx, int nrhs);

// X = U^{-1} L^{-1} P B for one large factored matrix; B (n x nrhs, ldb) is
// permuted into X (ldx), then solved in place.  perm from perm_from_ipiv_kernel.
template <typename T>
int bigtrs(cudaStream_t s, const T* LU, int lda, int n, const int* perm, const T* B, int ldb, T* X, int ldx,
           int nrhs, bool lower = true, bool upper = true);

int build_perm(cudaStream_t s, const int* ipiv, int n, int* perm);
int build_perm_batched(cudaStream_t s, const int* ipiv, long long strideP, int n, int batch, int* perm,
                       long long strideQ);

// Batched X = U^{-1} L^{-1} P B with the warp kernel (nrhs <= 4); perm from
// build_perm_batched.  Returns SLAB_ERR_ARG when the shape does not fit.
template <typename T>
int getrs_small(cudaStream_t s, int n, int nrhs, const T* LU, const long long* offLU, long long strideLU, int lda,
                const int* perm, const long long* offP, long long strideP, T* B, const long long* offB,
                long long strideB, int ldb, int batch);

// Batched X = U^{-1} L^{-1} P B for many right-hand sides (getrs_many_kernel,
// n <= 1024); perm from build_perm_batched.
template <typename T>
int getrs_many(cudaStream_t s, int n, int nrhs, const T* LU, long long strideLU, int lda, const int* perm,
               long long strideP, T* B, long long strideB, int ldb, int batch);
// Whether getrs_many's tile of n rows fits the device's shared memory.
template <typename T>
bool getrs_many_fits(int n);

// X = U^{-1} L^{-1} P B for one large factored matrix, nrhs <= 8, cooperative
// launch; Linv/Uinv from tri_inv_blocks with block size bs.
template <typename T>
int trsv_coop(cudaStream_t s, const T* LU, int lda, int n, const int* perm, const T* Linv, const T* Uinv, int bs,
              const T* B, int ldb, T* X, int ldx, int nrhs, bool trans = false);

// One panel step of biglu: factor columns k0..k0+nb (rows k0..n) with partial
// pivoting and apply its interchanges to every other column.  linv (nb x nb,
// may be null) receives the inverse of the unit-lower panel triangle when
// *linv_done comes back true.
template <typename T>
int biglu_panel_swap(cudaStream_t s, T* A, int lda, int n, int k0, int nb, int* ipiv, int* info, T* linv,
                     bool* linv_done);

// Panel factorization of columns [k0, k0+nb) (as biglu_panel_swap) with the
// interchanges applied only to the columns [c_lo, c_hi) outside the panel.
template <typename T>
int biglu_panel_swap_range(cudaStream_t s, T* A, int lda, int n, int k0, int nb, int c_lo, int c_hi, int* ipiv,
                           int* info, T* linv, bool* linv_done);

// Interchanges ipiv[k0 .. k0+npiv) (npiv <= 256) applied to the columns
// [lo1, hi1) and [lo2, hi2) of the n-row matrix A through a gather; perm:
// 1 + 2 * kRowpermMax ints of scratch.
template <typename T>
int laswp_gather(cudaStream_t s, T* A, int lda, int n, int k0, int npiv, const int* ipiv, int lo1, int hi1, int lo2,
                 int hi2, int* perm);

// X[k0:k0+nb, 0:ncols] = Inv X[k0:k0+nb, 0:ncols] with Inv a bs x bs inverted
// diagonal triangle (tri_inv_blocks layout, column-major, ld bs).
template <typename T>
int trsm_inv(cudaStream_t s, const T* Inv, int bs, int k0, int nb, T* X, int ldx, int ncols);

// Same contract as trsv_coop with bs = 64, run by one thread-block cluster.
// Returns SLAB_ERR_ARG when the shape does not fit (caller falls back).
template <typename T>
int trsv_cluster(cudaStream_t s, const T* LU, int lda, int n, const int* perm, const T* Linv, const T* Uinv,
                 const T* B, int ldb, T* X, int ldx, int nrhs, bool trans = false);

// C = beta C + alpha A^T B (A is k x m); same batching conventions as gemm.
template <typename T>
int gemm_tn(cudaStream_t s, int m, int n, int k, T alpha, const T* A, const long long* offA, long long strideA,
            int lda, const T* B, const long long* offB, long long strideB, int ldb, T beta, T* C,
            const long long* offC, long long strideC, int ldc, int batch);

// Batched X = A^{-T} B with the warp kernel (nrhs <= 4).
template <typename T>
int getrs_small_t(cudaStream_t s, int n, int nrhs, const T* LU, const long long* offLU, long long strideLU, int lda,
                  const int* perm, const long long* offP, long long strideP, T* B, const long long* offB,
                  long long strideB, int ldb, int batch);

size_t smem_limit_bytes();

// Raise a kernel's dynamic shared-memory limit to the device maximum (minus its
// static shared memory), once.  The limit is never lowered: CUDA graphs that
// captured a larger launch stay valid.  Returns the dynamic bytes allowed.
size_t allow_dynamic_smem(const void* kernel);

template <typename K>
int ensure_smem(K* kernel, size_t bytes, const char* what) {
  const size_t lim = allow_dynamic_smem(reinterpret_cast<const void*>(kernel));
  if (bytes > lim) return set_error(SLAB_ERR_ARG, "%s needs %zu bytes of shared memory (limit %zu)", what, bytes, lim);
  return SLAB_OK;
}

}  // namespace slab
