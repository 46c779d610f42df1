// FP64 matrix products on the BF16 tensor cores (tcgen05) by exact slicing.
//
// C = alpha A B + beta C with A (m x k), B (k x n), C column-major FP64.
// Every row of A and column of B is scaled by a power of two so that its
// largest entry is below 1, read as a 56-bit fixed-point integer (integer
// operations on the IEEE bit pattern; rounding error <= 2^-57 of the row or
// column maximum) and cut into eight 7-bit slices, each an integer in
// [-127, 127] held exactly in BF16:
//     A = diag(2^e) sum_s 2^(-7s) A_s,   B = sum_t 2^(-7t) B_t diag(2^f).
// The products A_s B_t with s + t <= 9 (36 of them) run on the tensor cores
// with FP32 accumulation in tensor memory.  Over a K chunk of 128 a product
// sum is an integer below 128 * 127^2 < 2^21, and the (at most eight)
// products of one weight 2^(-7(s+t)) share one accumulator (< 2^24), so every
// FP32 accumulation is exact.  The eight level accumulators of a 128 x 32
// output tile sit in consecutive tensor-memory columns, level s + t at
// columns 32 (s + t - 2): with the eight B slices stacked in shared memory,
// one MMA of width N = 32 (9 - s) computes A_s B_t for every t <= 9 - s at
// once, each 32-column block landing on its own level.  The epilogue warps
// drain the levels into two 64-bit integer fixed-point sums per output
// (levels 2-5 and 6-9), so the
// FP64 pipe -- a small fraction of the FP32 rate on GB300 -- only does the
// final combination, scaling and alpha/beta update (about six FP64 operations
// per output).  The dropped levels s + t >= 10 and the fixed-point rounding
// bound the error by about k 2^-53 max|A_i.| max|B_.j|, the size of the
// worst-case bound of an FP64 dot product.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdint>
#include <mutex>

#include "common.cuh"
#include "dense.cuh"
#include "ozaki.cuh"
#include "tc.cuh"

namespace slab {

namespace {

constexpr int kSl = 8;         // slices per operand
constexpr int kSliceBits = 7;  // bits per slice
constexpr int kBM = 128, kBN = 32, kBK = 64, kChunk = 128;
constexpr int kGroups = 8;  // one accumulator per level s + t = 2..9
// Shared-memory rings: one A slice tile per (K step, slice) and all eight B
// slice tiles of a K step together, so each B slice is loaded once per K step
// (not once per A slice it pairs with).
constexpr int kAStages = 6;
constexpr int kBStages = 3;
constexpr int kAbytes = kBM * kBK * 2;
constexpr int kBbytes = kBN * kBK * 2;
constexpr int kBStageBytes = kSl * kBbytes;
constexpr int kNonFinite = INT_MIN;
// Two sets of the eight level accumulators: the MMAs of K chunk c + 1 run into
// one while the epilogue drains chunk c from the other.
constexpr int kAccCols = kGroups * kBN;
constexpr int kTmemCols = 2 * kAccCols;
constexpr size_t kGemmSmem = (size_t)kAStages * kAbytes + (size_t)kBStages * kBStageBytes + 1024 + 256;

static_assert(kTmemCols <= 512, "both accumulator sets must fit tensor memory");
static_assert(kSl * kBN <= 256, "one MMA covers all B slices of an A slice (N <= 256)");

__device__ __forceinline__ int biased_exp(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7FF);
}

// Power-of-two scale exponent of a row or column from its largest biased
// exponent (zeros and subnormals count as exponent 1); kNonFinite for Inf/NaN.
__device__ __forceinline__ int scale_of(int emax) {
  if (emax >= 2047) return kNonFinite;
  return (emax < 1 ? 1 : emax) - 1022;  // |x| < 2^scale for every entry
}

// 56-bit fixed-point magnitude of x relative to 2^scale (scale from scale_of),
// rounded to nearest (ties up): |x| 2^(56 - scale) < 2^56, so the result stays
// below 2^56 for every entry of the row or column.
__device__ __forceinline__ unsigned long long fixed56(double x, int scale) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int E = (int)((b >> 52) & 0x7FF);
  const unsigned long long mant = (b & 0xFFFFFFFFFFFFFull) | (E != 0 ? (1ull << 52) : 0ull);
  const int shift = (E < 1 ? 1 : E) - (scale + 1022) + 3;  // <= 3
  if (shift >= 0) return mant << shift;
  if (-shift > 54) return 0ull;
  return (mant + (1ull << (-shift - 1))) >> (-shift);
}

__device__ __forceinline__ __nv_bfloat16 slice_val(unsigned long long q, int s, bool neg) {
  const int d = (int)((q >> (56 - kSliceBits * (s + 1))) & 127ull);
  return __float2bfloat16_rn((float)(neg ? -d : d));
}

__global__ void rowmax_exp_kernel(const double* __restrict__ A, int lda, int m, int k, int* __restrict__ emax) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const int k0 = blockIdx.y * 64, k1 = min(k, k0 + 64);
  int e = 0;
  for (int kk = k0; kk < k1; ++kk) e = max(e, biased_exp(A[i + (size_t)kk * lda]));
  atomicMax(&emax[i], e);
}

__global__ void finish_scale_kernel(int* __restrict__ e, int m) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) e[i] = scale_of(e[i]);
}

// A (m x k, column-major) -> slices [s][i][kk] (K contiguous, row length kp),
// through a 32 x 32 shared-memory transpose.  Columns k..kp-1 are zero.
__global__ void __launch_bounds__(256) slice_a_kernel(const double* __restrict__ A, int lda, int m, int k, int kp,
                                                      const int* __restrict__ ea, __nv_bfloat16* __restrict__ out) {
  __shared__ __nv_bfloat16 t[kSl][32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int i0 = blockIdx.x * 32, kk0 = blockIdx.y * 32;
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + tx, kk = kk0 + r;
    double x = 0.0;
    int sc = 0;
    if (i < m) {
      sc = ea[i];
      if (kk < k) x = A[i + (size_t)kk * lda];
    }
    const bool bad = sc == kNonFinite;
    const unsigned long long q = bad ? 0ull : fixed56(x, sc);
    const bool neg = x < 0.0;
#pragma unroll
    for (int s = 0; s < kSl; ++s) t[s][r][tx] = slice_val(q, s, neg);
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + r, kk = kk0 + tx;
    if (i >= m || kk >= kp) continue;
#pragma unroll
    for (int s = 0; s < kSl; ++s) out[((size_t)s * m + i) * kp + kk] = t[s][tx][r];
  }
}

// B (k x n, column-major) -> slices [t][j][kk]; one warp per column, which also
// computes the column's scale exponent.
__global__ void __launch_bounds__(256) slice_b_kernel(const double* __restrict__ B, int ldb, int n, int k, int kp,
                                                      int* __restrict__ fb, __nv_bfloat16* __restrict__ out) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n) return;
  const double* col = B + (size_t)warp * ldb;
  int e = 0;
  for (int kk = lane; kk < k; kk += 32) e = max(e, biased_exp(col[kk]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
  const int sc = scale_of(e);
  if (lane == 0) fb[warp] = sc;
  for (int kk = lane; kk < kp; kk += 32) {
    const double x = kk < k ? col[kk] : 0.0;
    const unsigned long long q = sc == kNonFinite ? 0ull : fixed56(x, sc);
    const bool neg = x < 0.0;
#pragma unroll
    for (int s = 0; s < kSl; ++s) out[((size_t)s * n + warp) * kp + kk] = slice_val(q, s, neg);
  }
}

struct EmuArgs {
  int m, n, kp;
  double alpha, beta;
  double* C;
  int ldc;
  const int* ea;
  const int* fb;
  int* err;
};

__device__ __forceinline__ double pow2i(int e) {  // e in [-1022, 1023]
  return __longlong_as_double((long long)(e + 1023) << 52);
}

// Wait used on the way out: only the time limit ends it.
__device__ __forceinline__ void final_wait(uint64_t* bar, uint32_t parity, int* err) {
  const unsigned long long t0 = tc::globaltimer();
  while (!tc::mbar_try_wait(bar, parity)) {
    if (tc::globaltimer() - t0 > tc::kWaitNs) {
      atomicCAS(err, 0, 9);
      return;
    }
  }
}

// grid (ceil(m/128), ceil(n/32)), 192 threads: warp 0 TMA producer, warp 1
// tensor-memory owner and MMA issuer, warps 2-5 epilogue (one output row per thread).
__global__ void __launch_bounds__(192, 1) ozaki_gemm_kernel(const __grid_constant__ CUtensorMap tmA,
                                                            const __grid_constant__ CUtensorMap tmB, EmuArgs a) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* aring =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* bring = aring + (size_t)kAStages * kAbytes;
  uint64_t* fullA = reinterpret_cast<uint64_t*>(bring + (size_t)kBStages * kBStageBytes);
  uint64_t* emptyA = fullA + kAStages;
  uint64_t* fullB = emptyA + kAStages;
  uint64_t* emptyB = fullB + kBStages;
  uint64_t* accf = emptyB + kBStages;  // [2]: chunk products complete in accumulator set b
  uint64_t* acce = accf + 2;           // [2]: accumulator set b drained
  uint64_t* fin = acce + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(fin + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i0 = blockIdx.x * kBM, j0 = blockIdx.y * kBN;
  const int nchunk = (a.kp + kChunk - 1) / kChunk;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kAStages; ++s) {
      tc::mbar_init(&fullA[s], 1);
      tc::mbar_init(&emptyA[s], 1);
    }
    for (int s = 0; s < kBStages; ++s) {
      tc::mbar_init(&fullB[s], 1);
      tc::mbar_init(&emptyB[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&accf[b], 1);
      tc::mbar_init(&acce[b], 128);
    }
    tc::mbar_init(fin, 1);
    tc::fence_mbar_init();
  }
  if (warp == 1) tc::tmem_alloc(tmem_slot, kTmemCols);
  if (warp == 0 && lane == 0) {
    tc::prefetch_tmap(&tmA);
    tc::prefetch_tmap(&tmB);
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tbase = *tmem_slot;

  // Order of work, shared by the producer and the MMA issuer: chunk c, K step
  // kb: the B block of (c, kb), then the A slices s0 = 0..7 of (c, kb).
  if (warp == 0) {
    if (lane == 0) {
      int lastA[kAStages], lastB[kBStages];
#pragma unroll
      for (int s = 0; s < kAStages; ++s) lastA[s] = -1;
#pragma unroll
      for (int s = 0; s < kBStages; ++s) lastB[s] = -1;
      int itA = 0, itB = 0;
      bool ok = true;
      for (int c = 0; c < nchunk && ok; ++c) {
        const int nkb = min(kChunk, a.kp - c * kChunk + kBK - 1) / kBK;
        for (int kb = 0; kb < nkb && ok; ++kb) {
          const int kx = c * kChunk + kb * kBK;
          {
            const int st = itB % kBStages, round = itB / kBStages;
            if (!tc::mbar_wait(&emptyB[st], (uint32_t)((round & 1) ^ 1), a.err, 1)) {
              ok = false;
              break;
            }
            tc::mbar_arrive_expect_tx(&fullB[st], (uint32_t)kBStageBytes);
            unsigned char* bp = bring + (size_t)st * kBStageBytes;
            for (int t0 = 0; t0 < kSl; ++t0) tc::tma_load_3d(bp + t0 * kBbytes, &tmB, &fullB[st], kx, j0, t0);
            lastB[st] = round;
            ++itB;
          }
          for (int s0 = 0; s0 < kSl; ++s0) {
            const int st = itA % kAStages, round = itA / kAStages;
            if (!tc::mbar_wait(&emptyA[st], (uint32_t)((round & 1) ^ 1), a.err, 1)) {
              ok = false;
              break;
            }
            tc::mbar_arrive_expect_tx(&fullA[st], (uint32_t)kAbytes);
            tc::tma_load_3d(aring + (size_t)st * kAbytes, &tmA, &fullA[st], kx, i0, s0);
            lastA[st] = round;
            ++itA;
          }
        }
      }
      // no copy may still be in flight when the CTA leaves
      for (int s = 0; s < kAStages; ++s)
        if (lastA[s] >= 0) final_wait(&fullA[s], (uint32_t)(lastA[s] & 1), a.err);
      for (int s = 0; s < kBStages; ++s)
        if (lastB[s] >= 0) final_wait(&fullB[s], (uint32_t)(lastB[s] & 1), a.err);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int itA = 0, itB = 0;
      bool ok = true;
      for (int c = 0; c < nchunk && ok; ++c) {
        // accumulator set c & 1 was last used by chunk c - 2 (its ((c >> 1) - 1)-th drain)
        const int buf = c & 1;
        if (c >= 2) {
          if (!tc::mbar_wait(&acce[buf], (uint32_t)(((c >> 1) - 1) & 1), a.err, 3)) break;
          tc::tc_fence_after();
        }
        const int nkb = min(kChunk, a.kp - c * kChunk + kBK - 1) / kBK;
        for (int kb = 0; kb < nkb && ok; ++kb) {
          const int stB = itB % kBStages, roundB = itB / kBStages;
          if (!tc::mbar_wait(&fullB[stB], (uint32_t)(roundB & 1), a.err, 4)) {
            ok = false;
            break;
          }
          // descriptors are built once per stage; a 32-byte K step and a B
          // tile step only add to the start-address field (address >> 4)
          const uint64_t bdesc0 = tc::sdesc_kmajor_sw128(tc::smem_u32(bring + (size_t)stB * kBStageBytes));
          for (int s0 = 0; s0 < kSl; ++s0) {
            const int stA = itA % kAStages, roundA = itA / kAStages;
            if (!tc::mbar_wait(&fullA[stA], (uint32_t)(roundA & 1), a.err, 4)) {
              ok = false;
              break;
            }
            tc::tc_fence_after();
            const uint64_t adesc = tc::sdesc_kmajor_sw128(tc::smem_u32(aring + (size_t)stA * kAbytes));
            // A_s0 against B slices 0 .. 7-s0 (rows 0 .. 32 (8-s0) - 1 of the B block):
            // block t0 of the result is level s0 + t0 + 2, at column 32 (s0 + t0)
            const uint32_t idesc = tc::idesc_bf16_f32(kBM, kBN * (kSl - s0));
            const uint32_t dcol = tbase + (uint32_t)(buf * kAccCols + kBN * s0);
            // the chunk's first MMA (s0 = 0 spans every level) starts the accumulators
            tc::mma_bf16(dcol, adesc, bdesc0, idesc, (kb == 0 && s0 == 0) ? 0u : 1u);
#pragma unroll
            for (int kk = 1; kk < kBK / 16; ++kk)
              tc::mma_bf16(dcol, adesc + (uint64_t)(2 * kk), bdesc0 + (uint64_t)(2 * kk), idesc, 1u);
            tc::mma_commit(&emptyA[stA]);  // the A slot is free once these products complete
            ++itA;
          }
          if (ok) tc::mma_commit(&emptyB[stB]);  // and the B block after the last slice of this step
          ++itB;
        }
        if (ok) tc::mma_commit(&accf[buf]);
      }
      tc::mma_commit(fin);  // every product issued has completed before tensor memory is released
      final_wait(fin, 0, a.err);
    }
  } else {
    const int q = warp & 3;  // tensor-memory lane quarter of this warp
    const int row = q * 32 + lane;
    long long hi[kBN], lo[kBN];
#pragma unroll
    for (int j = 0; j < kBN; ++j) hi[j] = lo[j] = 0;
    bool ok = true;
    for (int c = 0; c < nchunk; ++c) {
      const int buf = c & 1;
      if (!tc::mbar_wait(&accf[buf], (uint32_t)((c >> 1) & 1), a.err, 5)) {
        ok = false;
        break;
      }
      tc::tc_fence_after();
#pragma unroll 1
      for (int g = 0; g < kGroups; ++g) {
        uint32_t r[32];
        tc::tmem_ld_32x32b_x32(tbase + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * kAccCols + g * kBN), r);
        tc::tmem_ld_wait();
        const int L = g + 2;
        if (g < 4) {
          const int sh = 7 * (5 - L);
#pragma unroll
          for (int j = 0; j < kBN; ++j) hi[j] += (long long)__float2int_rz(__uint_as_float(r[j])) << sh;
        } else {
          const int sh = 7 * (9 - L);
#pragma unroll
          for (int j = 0; j < kBN; ++j) lo[j] += (long long)__float2int_rz(__uint_as_float(r[j])) << sh;
        }
      }
      tc::tc_fence_before();
      tc::mbar_arrive(&acce[buf]);
    }
    if (ok && *reinterpret_cast<volatile int*>(a.err) == 0) {
      const int i = i0 + row;
      if (i < a.m) {
        const int ei = a.ea[i];
        const double w_hi = pow2i(-35), w_lo = pow2i(-63);
#pragma unroll
        for (int j = 0; j < kBN; ++j) {
          const int jj = j0 + j;
          if (jj >= a.n) break;
          const int fj = a.fb[jj];
          double v;
          if (ei == kNonFinite || fj == kNonFinite) {
            v = __longlong_as_double(0x7FF8000000000000ll);
          } else {
            v = (double)hi[j] * w_hi + (double)lo[j] * w_lo;
            const int e = ei + fj, e1 = e / 2;
            v = v * pow2i(e1) * pow2i(e - e1);
          }
          double* cp = a.C + i + (size_t)jj * a.ldc;
          *cp = a.beta == 0.0 ? a.alpha * v : a.alpha * v + a.beta * *cp;
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tbase, kTmemCols);
  }
}

using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encode_fn() {
  static std::once_flag once;
  static EncodeFn fn = nullptr;
  std::call_once(once, []() {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeFn>(p);
    cudaGetLastError();
  });
  return fn;
}

// 3-D map over slices [S][rows][kp] (bf16), box {64, box_rows, 1}, 128-byte swizzle.
int make_slice_map(CUtensorMap* map, const void* base, int kp, int rows, int box_rows) {
  EncodeFn fn = encode_fn();
  if (!fn) return set_error(SLAB_ERR_CUDA, "tensor-map encoder unavailable");
  const cuuint64_t dims[3] = {(cuuint64_t)kp, (cuuint64_t)rows, (cuuint64_t)kSl};
  const cuuint64_t strides[2] = {(cuuint64_t)kp * 2, (cuuint64_t)rows * kp * 2};
  const cuuint32_t box[3] = {(cuuint32_t)kBK, (cuuint32_t)box_rows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(SLAB_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return SLAB_OK;
}

size_t al256(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace

size_t dgemm_emu_work_bytes(int m, int n, int k) {
  if (m <= 0 || n <= 0 || k <= 0) return 256;
  const size_t kp = (size_t)round_up(k, 8);
  return al256(sizeof(int)) + al256((size_t)kSl * m * kp * 2) + al256((size_t)kSl * n * kp * 2) +
         al256((size_t)m * sizeof(int)) + al256((size_t)n * sizeof(int));
}

int dgemm_emu(cudaStream_t s, int m, int n, int k, double alpha, const double* A, int lda, const double* B, int ldb,
              double beta, double* C, int ldc, void* work, size_t work_bytes, int* err) {
  if (m <= 0 || n <= 0) return SLAB_OK;
  if (k <= 0 || !A || !B || !C || !work || !err || lda < m || ldb < k || ldc < m)
    return set_error(SLAB_ERR_ARG, "dgemm_emu: invalid arguments");
  if (work_bytes < dgemm_emu_work_bytes(m, n, k)) return set_error(SLAB_ERR_ARG, "dgemm_emu: work buffer too small");
  const int kp = round_up(k, 8);
  unsigned char* w = static_cast<unsigned char*>(work);
  w += al256(sizeof(int));  // first slot reserved for the caller's use
  __nv_bfloat16* Asl = reinterpret_cast<__nv_bfloat16*>(w);
  w += al256((size_t)kSl * m * kp * 2);
  __nv_bfloat16* Bsl = reinterpret_cast<__nv_bfloat16*>(w);
  w += al256((size_t)kSl * n * kp * 2);
  int* ea = reinterpret_cast<int*>(w);
  w += al256((size_t)m * sizeof(int));
  int* fb = reinterpret_cast<int*>(w);
  SLAB_CUDA_TRY(cudaMemsetAsync(ea, 0, (size_t)m * sizeof(int), s));
  rowmax_exp_kernel<<<dim3(ceil_div(m, 256), ceil_div(k, 64)), 256, 0, s>>>(A, lda, m, k, ea);
  SLAB_CHECK_LAUNCH();
  finish_scale_kernel<<<ceil_div(m, 256), 256, 0, s>>>(ea, m);
  SLAB_CHECK_LAUNCH();
  slice_a_kernel<<<dim3(ceil_div(m, 32), ceil_div(kp, 32)), 256, 0, s>>>(A, lda, m, k, kp, ea, Asl);
  SLAB_CHECK_LAUNCH();
  slice_b_kernel<<<ceil_div(n * 32, 256), 256, 0, s>>>(B, ldb, n, k, kp, fb, Bsl);
  SLAB_CHECK_LAUNCH();
  CUtensorMap tmA, tmB;
  SLAB_TRY(make_slice_map(&tmA, Asl, kp, m, kBM));
  SLAB_TRY(make_slice_map(&tmB, Bsl, kp, n, kBN));
  SLAB_TRY(ensure_smem(ozaki_gemm_kernel, kGemmSmem, "dgemm_emu"));
  EmuArgs ea_{m, n, kp, alpha, beta, C, ldc, ea, fb, err};
  ozaki_gemm_kernel<<<dim3(ceil_div(m, kBM), ceil_div(n, kBN)), 192, kGemmSmem, s>>>(tmA, tmB, ea_);
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}

int bigtrs_inv_emu(cudaStream_t s, const double* LU, int lda, int n, const int* perm, const double* Linv,
                   const double* Uinv, int bs, const double* B, int ldb, double* X, int ldx, int nrhs,
                   const EmuWork& w) {
  if (n <= 0 || nrhs <= 0) return SLAB_OK;
  if (kEmuOuter % bs != 0) return set_error(SLAB_ERR_ARG, "bigtrs_inv_emu: block size %d does not divide %d", bs, kEmuOuter);
  const long long tot = (long long)n * nrhs;
  permute_rows_kernel<double><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(B, ldb, X, ldx, n, nrhs, perm);
  SLAB_CHECK_LAUNCH();
  for (int ob0 = 0; ob0 < n; ob0 += kEmuOuter) {
    const int obe = n - ob0 < kEmuOuter ? n : ob0 + kEmuOuter;
    for (int k0 = ob0; k0 < obe; k0 += bs) {
      const int nb = obe - k0 < bs ? obe - k0 : bs;
      SLAB_TRY(trsm_inv<double>(s, Linv + (size_t)(k0 / bs) * bs * bs, bs, k0, nb, X, ldx, nrhs));
      const int inner = obe - k0 - nb;
      if (inner > 0)
        SLAB_TRY(gemm<double>(s, inner, nrhs, nb, -1.0, LU + (size_t)k0 * lda + k0 + nb, nullptr, 0, lda, X + k0,
                              nullptr, 0, ldx, 1.0, X + k0 + nb, nullptr, 0, ldx, 1));
    }
    const int rest = n - obe;
    if (rest > 0)
      SLAB_TRY(dgemm_emu(s, rest, nrhs, obe - ob0, -1.0, LU + (size_t)ob0 * lda + obe, lda, X + ob0, ldx, 1.0,
                         X + obe, ldx, w.buf, w.bytes, w.err));
  }
  for (int ob0 = ((n - 1) / kEmuOuter) * kEmuOuter; ob0 >= 0; ob0 -= kEmuOuter) {
    const int obe = n - ob0 < kEmuOuter ? n : ob0 + kEmuOuter;
    for (int k0 = ((obe - 1 - ob0) / bs) * bs + ob0; k0 >= ob0; k0 -= bs) {
      const int nb = obe - k0 < bs ? obe - k0 : bs;
      SLAB_TRY(trsm_inv<double>(s, Uinv + (size_t)(k0 / bs) * bs * bs, bs, k0, nb, X, ldx, nrhs));
      const int inner = k0 - ob0;
      if (inner > 0)
        SLAB_TRY(gemm<double>(s, inner, nrhs, nb, -1.0, LU + (size_t)k0 * lda + ob0, nullptr, 0, lda, X + k0, nullptr,
                              0, ldx, 1.0, X + ob0, nullptr, 0, ldx, 1));
    }
    if (ob0 > 0)
      SLAB_TRY(dgemm_emu(s, ob0, nrhs, obe - ob0, -1.0, LU + (size_t)ob0 * lda, lda, X + ob0, ldx, 1.0, X, ldx, w.buf,
                         w.bytes, w.err));
  }
  return SLAB_OK;
}

namespace {
// Block (r, c) of size kB of an outer block's inverse, ld kEmuOuter.
constexpr int kOB = kEmuOuter;

// Copies the 64 x 64 diagonal inverses into their places in the outer blocks
// (grid: one CTA per 64-row block; blocks past n are left zero).
__global__ void place_diag_inv_kernel(const double* __restrict__ Inv64, int nblk64, double* __restrict__ Out) {
  const int k = blockIdx.x;
  if (k >= nblk64) return;
  const int ob = k / (kOB / 64), i0 = (k % (kOB / 64)) * 64;
  double* O = Out + (size_t)ob * kOB * kOB;
  const double* I = Inv64 + (size_t)k * 64 * 64;
  for (int idx = threadIdx.x; idx < 64 * 64; idx += blockDim.x) {
    const int r = idx % 64, c = idx / 64;
    O[(size_t)(i0 + c) * kOB + i0 + r] = I[idx];
  }
}
}  // namespace

size_t outer_tri_tmp_elems(int n) {
  const int nob = (n + kOB - 1) / kOB;
  return (size_t)nob * 128 * 128;
}

// One doubling step for every outer block, halves [base, base + sa) and
// [base + sa, base + sa + sc) of each (sa = sc = h for the full blocks).
// lower: O = -C^{-1} (B A^{-1}) with B = L[below, left]; upper: O = -A^{-1} (B C^{-1})
// with B = U[above, right].  The full outer blocks go as one batched product,
// the last (partial) outer block on its own with its true sizes.
static int doubling_step(cudaStream_t s, const double* LU, int lda, int n, double* Inv, double* tmp, int h, int base,
                         bool upper) {
  const int nob = (n + kOB - 1) / kOB;
  const int nfull = n / kOB;
  const long long sLU = (long long)kOB * lda + kOB, sInv = (long long)kOB * kOB, sT = 128LL * 128;
  auto step = [&](int count, int ob0, int sa, int sc) -> int {
    if (count <= 0 || sa <= 0 || sc <= 0) return SLAB_OK;
    const long long r0 = (long long)ob0 * kOB + base;
    double* I0 = Inv + (size_t)ob0 * sInv;
    const double* Ai = I0 + (size_t)base * kOB + base;              // sa x sa
    const double* Ci = I0 + (size_t)(base + sa) * kOB + base + sa;   // sc x sc
    if (!upper) {
      const double* B = LU + (size_t)r0 * lda + r0 + sa;              // L[r0+sa.., r0..]: sc x sa
      double* O = I0 + (size_t)base * kOB + base + sa;                // rows base+sa.., cols base..
      SLAB_TRY(gemm<double>(s, sc, sa, sa, 1.0, B, nullptr, sLU, lda, Ai, nullptr, sInv, kOB, 0.0, tmp, nullptr, sT,
                            sc, count));
      SLAB_TRY(gemm<double>(s, sc, sa, sc, -1.0, Ci, nullptr, sInv, kOB, tmp, nullptr, sT, sc, 0.0, O, nullptr, sInv,
                            kOB, count));
    } else {
      const double* B = LU + (size_t)(r0 + sa) * lda + r0;            // U[r0.., r0+sa..]: sa x sc
      double* O = I0 + (size_t)(base + sa) * kOB + base;              // rows base.., cols base+sa..
      SLAB_TRY(gemm<double>(s, sa, sc, sc, 1.0, B, nullptr, sLU, lda, Ci, nullptr, sInv, kOB, 0.0, tmp, nullptr, sT,
                            sa, count));
      SLAB_TRY(gemm<double>(s, sa, sc, sa, -1.0, Ai, nullptr, sInv, kOB, tmp, nullptr, sT, sa, 0.0, O, nullptr, sInv,
                            kOB, count));
    }
    return SLAB_OK;
  };
  SLAB_TRY(step(nfull, 0, h, h));
  if (nob > nfull) {  // last outer block, rows [nfull*kOB, n)
    const int nb = n - nfull * kOB;
    const int sa = std::min(h, nb - base), sc = std::min(h, nb - base - h);
    SLAB_TRY(step(1, nfull, sa, sc));
  }
  return SLAB_OK;
}

int outer_tri_inverses(cudaStream_t s, const double* LU, int lda, int n, const double* Linv64, const double* Uinv64,
                       double* LoInv, double* UoInv, double* tmp) {
  static_assert(kEmuOuter == 256, "two doubling steps from 64-row blocks");
  if (n <= 0) return SLAB_OK;
  const int nob = (n + kOB - 1) / kOB, nblk64 = (n + 63) / 64;
  for (double* Inv : {LoInv, UoInv}) SLAB_CUDA_TRY(cudaMemsetAsync(Inv, 0, (size_t)nob * kOB * kOB * 8, s));
  place_diag_inv_kernel<<<nblk64, 256, 0, s>>>(Linv64, nblk64, LoInv);
  SLAB_CHECK_LAUNCH();
  place_diag_inv_kernel<<<nblk64, 256, 0, s>>>(Uinv64, nblk64, UoInv);
  SLAB_CHECK_LAUNCH();
  for (int up = 0; up < 2; ++up) {
    double* Inv = up ? UoInv : LoInv;
    SLAB_TRY(doubling_step(s, LU, lda, n, Inv, tmp, 64, 0, up));
    SLAB_TRY(doubling_step(s, LU, lda, n, Inv, tmp, 64, 128, up));
    SLAB_TRY(doubling_step(s, LU, lda, n, Inv, tmp, 128, 0, up));
  }
  return SLAB_OK;
}

int bigtrs_outer_emu(cudaStream_t s, const double* LU, int lda, int n, const int* perm, const double* LoInv,
                     const double* UoInv, const double* B, int ldb, double* X, int ldx, int nrhs, double* Y,
                     const EmuWork& w) {
  if (n <= 0 || nrhs <= 0) return SLAB_OK;
  const long long tot = (long long)n * nrhs;
  permute_rows_kernel<double><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(B, ldb, X, ldx, n, nrhs, perm);
  SLAB_CHECK_LAUNCH();
  const int nob = (n + kOB - 1) / kOB;
  auto diag = [&](const double* Inv, int ob) -> int {
    const int ob0 = ob * kOB, nb = std::min(kOB, n - ob0);
    SLAB_TRY(dgemm_emu(s, nb, nrhs, nb, 1.0, Inv + (size_t)ob * kOB * kOB, kOB, X + ob0, ldx, 0.0, Y, kOB, w.buf,
                       w.bytes, w.err));
    SLAB_CUDA_TRY(cudaMemcpy2DAsync(X + ob0, (size_t)ldx * 8, Y, (size_t)kOB * 8, (size_t)nb * 8, nrhs,
                                    cudaMemcpyDeviceToDevice, s));
    return SLAB_OK;
  };
  for (int ob = 0; ob < nob; ++ob) {
    const int ob0 = ob * kOB, obe = std::min(n, ob0 + kOB);
    SLAB_TRY(diag(LoInv, ob));
    if (obe < n)
      SLAB_TRY(dgemm_emu(s, n - obe, nrhs, obe - ob0, -1.0, LU + (size_t)ob0 * lda + obe, lda, X + ob0, ldx, 1.0,
                         X + obe, ldx, w.buf, w.bytes, w.err));
  }
  for (int ob = nob - 1; ob >= 0; --ob) {
    const int ob0 = ob * kOB, obe = std::min(n, ob0 + kOB);
    SLAB_TRY(diag(UoInv, ob));
    if (ob0 > 0)
      SLAB_TRY(dgemm_emu(s, ob0, nrhs, obe - ob0, -1.0, LU + (size_t)ob0 * lda, lda, X + ob0, ldx, 1.0, X, ldx,
                         w.buf, w.bytes, w.err));
  }
  return SLAB_OK;
}

namespace {
// U12 = L11^{-1} A12 for the rows [ob0, obe) of the columns [c0, c0 + nc),
// then A22 -= A21 U12 below them on the tensor cores (blk_linv: inverted
// 64 x 64 diagonal triangles of the outer block's unit-lower L11).
int outer_update(cudaStream_t s, double* A, int lda, int n, int ob0, int obe, int c0, int nc, const double* blk_linv,
                 const EmuWork& w) {
  constexpr int kB = 64;
  if (nc <= 0) return SLAB_OK;
  double* A12 = A + (size_t)c0 * lda;
  for (int b0 = ob0; b0 < obe; b0 += kB) {
    const int bn = obe - b0 < kB ? obe - b0 : kB;
    SLAB_TRY(trsm_inv<double>(s, blk_linv + (size_t)((b0 - ob0) / kB) * kB * kB, kB, b0, bn, A12, lda, nc));
    const int below = obe - b0 - bn;
    if (below > 0)
      SLAB_TRY(gemm<double>(s, below, nc, bn, -1.0, A + (size_t)b0 * lda + b0 + bn, nullptr, 0, lda, A12 + b0,
                            nullptr, 0, lda, 1.0, A12 + b0 + bn, nullptr, 0, lda, 1));
  }
  return dgemm_emu(s, n - obe, nc, obe - ob0, -1.0, A + (size_t)ob0 * lda + obe, lda, A12 + ob0, lda, 1.0,
                   A12 + obe, lda, w.buf, w.bytes, w.err);
}
}  // namespace

int biglu_emu(cudaStream_t s, double* A, int lda, int n, int* ipiv, int* info, double* panel_linv, double* blk_linv,
              const EmuWork& w, const Lookahead* la) {
  constexpr int kB = 64;  // diagonal blocks of the outer triangular solve
  const bool look = la && la->side && la->fork && la->join && la->perm;
  bool side_busy = false;
  for (int ob0 = 0; ob0 < n; ob0 += kEmuOuter) {
    const int obe = n - ob0 < kEmuOuter ? n : ob0 + kEmuOuter;
    for (int k0 = ob0; k0 < obe; k0 += kNB) {
      const int nb = obe - k0 < kNB ? obe - k0 : kNB;
      bool linv_done = false;
      if (look)
        SLAB_TRY(biglu_panel_swap_range<double>(s, A, lda, n, k0, nb, ob0, obe, ipiv, info, panel_linv, &linv_done));
      else
        SLAB_TRY(biglu_panel_swap<double>(s, A, lda, n, k0, nb, ipiv, info, panel_linv, &linv_done));
      const int inner = obe - k0 - nb;
      if (inner > 0) {
        if (!linv_done) SLAB_TRY(tri_inv_blocks<double>(s, A + (size_t)k0 * lda + k0, lda, nb, kNB, panel_linv, nullptr));
        SLAB_TRY(trsm_inv<double>(s, panel_linv, linv_done ? nb : kNB, k0, nb, A + (size_t)(k0 + nb) * lda, lda,
                                  inner));
        SLAB_TRY(gemm<double>(s, n - k0 - nb, inner, nb, -1.0, A + (size_t)k0 * lda + k0 + nb, nullptr, 0, lda,
                              A + (size_t)(k0 + nb) * lda + k0, nullptr, 0, lda, 1.0,
                              A + (size_t)(k0 + nb) * lda + k0 + nb, nullptr, 0, lda, 1));
      }
    }
    const int rest = n - obe;
    if (look) {
      // the side stream's update of the previous outer block reads the columns
      // left of ob0 and writes those right of obe: it finishes before this
      // block's interchanges reach them
      if (side_busy) SLAB_CUDA_TRY(cudaStreamWaitEvent(s, la->join, 0));
      side_busy = false;
      SLAB_TRY(laswp_gather<double>(s, A, lda, n, ob0, obe - ob0, ipiv, 0, ob0, obe, n, la->perm));
    }
    if (rest > 0) {
      // U12 = L11^{-1} A12 over the outer block's rows, then A22 -= A21 U12 on the tensor cores
      SLAB_TRY(tri_inv_blocks<double>(s, A + (size_t)ob0 * lda + ob0, lda, obe - ob0, kB, blk_linv, nullptr));
      const int now = look ? (rest < kEmuOuter ? rest : kEmuOuter) : rest;  // columns the next outer block needs
      SLAB_TRY(outer_update(s, A, lda, n, ob0, obe, obe, now, blk_linv, w));
      if (now < rest) {
        SLAB_CUDA_TRY(cudaEventRecord(la->fork, s));
        SLAB_CUDA_TRY(cudaStreamWaitEvent(la->side, la->fork, 0));
        SLAB_TRY(outer_update(la->side, A, lda, n, ob0, obe, obe + now, rest - now, blk_linv, w));
        SLAB_CUDA_TRY(cudaEventRecord(la->join, la->side));
        side_busy = true;
      }
    }
  }
  if (side_busy) SLAB_CUDA_TRY(cudaStreamWaitEvent(s, la->join, 0));
  return SLAB_OK;
}

}  // namespace slab

extern "C" size_t slab_dgemm_emu_work_bytes(int m, int n, int k) { return slab::dgemm_emu_work_bytes(m, n, k); }

extern "C" int slab_dgemm_emu(int m, int n, int k, double alpha, const double* A, int lda, const double* B, int ldb,
                              double beta, double* C, int ldc, void* work, size_t work_bytes, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!work || work_bytes < slab::dgemm_emu_work_bytes(m, n, k))
    return slab::set_error(SLAB_ERR_ARG, "slab_dgemm_emu: work buffer too small");
  int* err = static_cast<int*>(work);  // the reserved first slot
  SLAB_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
  SLAB_TRY(slab::dgemm_emu(s, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, work, work_bytes, err));
  int h = 0;
  SLAB_CUDA_TRY(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  SLAB_CUDA_TRY(cudaStreamSynchronize(s));
  if (h != 0) return slab::set_error(SLAB_ERR_CUDA, "slab_dgemm_emu: tensor-core pipeline wait expired (code %d)", h);
  return SLAB_OK;
}
