// FP32 matrix products on the tensor cores by exact TF32 splitting.
//
// Every FP32 operand x is written as three TF32 values whose sum is x exactly:
//     x0 = tf32(x),  x1 = tf32(x - x0),  x2 = (x - x0) - x1
// (round to nearest; x - x0 has at most 13 significant bits and x2 at most 3,
// so each slice is a TF32 value and no bit of x is lost).  The product
// A B = sum_{s,t} A_s B_t keeps the six slice pairs with s + t <= 2; the pairs
// left out weigh at most 2^-33 of |A||B|, below the FP32 rounding of the
// accumulation.  The six products run as tcgen05 kind::tf32 MMAs (one thread
// issues them) on operand tiles that TMA copies into shared memory with the
// 128-byte swizzle, accumulating in FP32 in tensor memory; four epilogue warps
// read the accumulator with tcgen05.ld and apply alpha and beta.  Within a K
// step the pairs are added smallest weight first.
//
// The slices are prepared by two small kernels into the caller's work buffer,
// K contiguous and K padded with zeros to a multiple of 32:
//     A slices [s][b][i][kk],  B slices [s][b][j][kk].
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "common.cuh"
#include "dense.cuh"
#include "tc.cuh"
#include "tcgemm.cuh"

namespace slab {

namespace {

constexpr int kTBM = 128;   // output rows per CTA (tensor-memory lanes)
constexpr int kTBK = 32;    // K per stage: 32 FP32 = one 128-byte swizzle row
constexpr int kNSl = 3;     // slices per operand
constexpr int kTStages = 2;
constexpr int kSliceA = kTBM * kTBK * 4;

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void split3(float x, float& s0, float& s1, float& s2) {
  s0 = tf32_rna(x);
  const float r = x - s0;
  s1 = tf32_rna(r);
  s2 = r - s1;
}

// A (m x k, column-major, batch stride sA) -> slices [s][b][i][kk] (mp rows of
// length kp), through a 32 x 32 shared-memory transpose.  Columns k..kp-1 and
// rows m..mp-1 are zero.
__global__ void __launch_bounds__(256) split_a_kernel(const float* __restrict__ A, int lda, long long sA, int m, int mp,
                                                      int k, int kp, int batch, float* __restrict__ out) {
  __shared__ float t[kNSl][32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int i0 = blockIdx.x * 32, kk0 = blockIdx.y * 32, b = blockIdx.z;
  const float* Ab = A + (size_t)b * sA;
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + tx, kk = kk0 + r;
    const float x = (i < m && kk < k) ? Ab[i + (size_t)kk * lda] : 0.f;
    float s0, s1, s2;
    split3(x, s0, s1, s2);
    t[0][r][tx] = s0;
    t[1][r][tx] = s1;
    t[2][r][tx] = s2;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + r, kk = kk0 + tx;
    if (i >= mp || kk >= kp) continue;
#pragma unroll
    for (int s = 0; s < kNSl; ++s) out[(((size_t)s * batch + b) * mp + i) * kp + kk] = t[s][tx][r];
  }
}

// B (k x n, column-major, batch stride sB) -> slices [s][b][j][kk] (np_ rows of
// length kp; rows n..np_-1 and columns k..kp-1 are zero).
__global__ void __launch_bounds__(256) split_b_kernel(const float* __restrict__ B, int ldb, long long sB, int n, int np_,
                                                      int k, int kp, int batch, float* __restrict__ out) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (idx >= (long long)np_ * kp) return;
  const int kk = (int)(idx % kp), j = (int)(idx / kp);
  const float x = (kk < k && j < n) ? B[(size_t)b * sB + kk + (size_t)j * ldb] : 0.f;
  float s0, s1, s2;
  split3(x, s0, s1, s2);
  const size_t o = ((size_t)b * np_ + j) * kp + kk, slab = (size_t)batch * np_ * kp;
  out[o] = s0;
  out[o + slab] = s1;
  out[o + 2 * slab] = s2;
}

struct TfArgs {
  int m, n, kp, batch;
  float alpha, beta;
  float* C;
  int ldc;
  long long sC;
  int* err;
};

// Wait used on the way out: only the time limit ends it.
__device__ __forceinline__ void final_wait_tf(uint64_t* bar, uint32_t parity, int* err) {
  const unsigned long long t0 = tc::globaltimer();
  while (!tc::mbar_try_wait(bar, parity)) {
    if (tc::globaltimer() - t0 > tc::kWaitNs) {
      atomicCAS(err, 0, 9);
      return;
    }
  }
}

template <int BN>
constexpr size_t tf32s_smem_bytes() {
  return (size_t)kTStages * kNSl * (kSliceA + BN * kTBK * 4) + 1024 + 256;
}

// grid (ceil(m/128), ceil(n/BN), batch), 192 threads: warp 0 TMA producer,
// warp 1 tensor-memory owner and MMA issuer, warps 2-5 epilogue (one output
// row per thread).
template <int BN>
__global__ void __launch_bounds__(192, 1) tf32s_gemm_kernel(const __grid_constant__ CUtensorMap tmA,
                                                            const __grid_constant__ CUtensorMap tmB, TfArgs a) {
  constexpr int kSliceB = BN * kTBK * 4;
  constexpr int kStage = kNSl * (kSliceA + kSliceB);
  extern __shared__ unsigned char smem_raw[];
  unsigned char* ring =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(ring + (size_t)kTStages * kStage);
  uint64_t* empty = full + kTStages;
  uint64_t* accf = empty + kTStages;
  uint64_t* fin = accf + 1;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(fin + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i0 = blockIdx.x * kTBM, j0 = blockIdx.y * BN, b = blockIdx.z;
  const int nk = a.kp / kTBK;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kTStages; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(accf, 1);
    tc::mbar_init(fin, 1);
    tc::fence_mbar_init();
  }
  if (warp == 1) tc::tmem_alloc(tmem_slot, BN);
  if (warp == 0 && lane == 0) {
    tc::prefetch_tmap(&tmA);
    tc::prefetch_tmap(&tmB);
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tbase = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int last[kTStages];
#pragma unroll
      for (int s = 0; s < kTStages; ++s) last[s] = -1;
      for (int kb = 0; kb < nk; ++kb) {
        const int st = kb % kTStages, round = kb / kTStages;
        if (!tc::mbar_wait(&empty[st], (uint32_t)((round & 1) ^ 1), a.err, 1)) break;
        tc::mbar_arrive_expect_tx(&full[st], (uint32_t)kStage);
        unsigned char* sp = ring + (size_t)st * kStage;
#pragma unroll
        for (int sl = 0; sl < kNSl; ++sl) {
          tc::tma_load_3d(sp + sl * kSliceA, &tmA, &full[st], kb * kTBK, i0, sl * a.batch + b);
          tc::tma_load_3d(sp + kNSl * kSliceA + sl * kSliceB, &tmB, &full[st], kb * kTBK, j0, sl * a.batch + b);
        }
        last[st] = round;
      }
      // no copy may still be in flight when the CTA leaves
      for (int s = 0; s < kTStages; ++s)
        if (last[s] >= 0) final_wait_tf(&full[s], (uint32_t)(last[s] & 1), a.err);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = tc::idesc_tf32_f32(kTBM, BN);
      bool ok = true;
      for (int kb = 0; kb < nk; ++kb) {
        const int st = kb % kTStages, round = kb / kTStages;
        if (!tc::mbar_wait(&full[st], (uint32_t)(round & 1), a.err, 2)) {
          ok = false;
          break;
        }
        tc::tc_fence_after();
        unsigned char* sp = ring + (size_t)st * kStage;
        uint64_t ad[kNSl], bd[kNSl];
#pragma unroll
        for (int sl = 0; sl < kNSl; ++sl) {
          ad[sl] = tc::sdesc_kmajor_sw128(tc::smem_u32(sp + sl * kSliceA));
          bd[sl] = tc::sdesc_kmajor_sw128(tc::smem_u32(sp + kNSl * kSliceA + sl * kSliceB));
        }
        // a K step of 8 TF32 values is 32 bytes: 2 in the start-address field
#pragma unroll
        for (int kk = 0; kk < kTBK / 8; ++kk) {
          const uint64_t o = (uint64_t)(2 * kk);
          tc::mma_tf32(tbase, ad[2] + o, bd[0] + o, idesc, (kb | kk) ? 1u : 0u);
          tc::mma_tf32(tbase, ad[1] + o, bd[1] + o, idesc, 1u);
          tc::mma_tf32(tbase, ad[0] + o, bd[2] + o, idesc, 1u);
          tc::mma_tf32(tbase, ad[1] + o, bd[0] + o, idesc, 1u);
          tc::mma_tf32(tbase, ad[0] + o, bd[1] + o, idesc, 1u);
          tc::mma_tf32(tbase, ad[0] + o, bd[0] + o, idesc, 1u);
        }
        tc::mma_commit(&empty[st]);  // the stage is free once these products complete
      }
      if (ok) tc::mma_commit(accf);
      tc::mma_commit(fin);  // every product issued has completed before tensor memory is released
      final_wait_tf(fin, 0, a.err);
    }
  } else {
    const int q = warp & 3;  // tensor-memory lane quarter of this warp
    const int i = i0 + q * 32 + lane;
    if (tc::mbar_wait(accf, 0, a.err, 3)) {
      tc::tc_fence_after();
      float* Cb = a.C + (size_t)b * a.sC;
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
        uint32_t r[32];
        tc::tmem_ld_32x32b_x32(tbase + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, r);
        tc::tmem_ld_wait();
        const int ncol = a.n - (j0 + c0);
        if (ncol <= 0 || i >= a.m) continue;
        float* cp = Cb + i + (size_t)(j0 + c0) * a.ldc;
        if (a.beta != 0.f) {
          float cv[32];
#pragma unroll
          for (int c = 0; c < 32; ++c) cv[c] = c < ncol ? cp[(size_t)c * a.ldc] : 0.f;
#pragma unroll
          for (int c = 0; c < 32; ++c)
            if (c < ncol) cp[(size_t)c * a.ldc] = a.alpha * __uint_as_float(r[c]) + a.beta * cv[c];
        } else {
#pragma unroll
          for (int c = 0; c < 32; ++c)
            if (c < ncol) cp[(size_t)c * a.ldc] = a.alpha * __uint_as_float(r[c]);
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tbase, BN);
  }
}

using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encode_fn_tf() {
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

// 3-D map over FP32 slices [depth][rows][kp], box {32, box_rows, 1}, 128-byte swizzle.
int make_f32_map(CUtensorMap* map, const void* base, int kp, int rows, int depth, int box_rows) {
  EncodeFn fn = encode_fn_tf();
  if (!fn) return set_error(SLAB_ERR_CUDA, "tensor-map encoder unavailable");
  const cuuint64_t dims[3] = {(cuuint64_t)kp, (cuuint64_t)rows, (cuuint64_t)depth};
  const cuuint64_t strides[2] = {(cuuint64_t)kp * 4, (cuuint64_t)rows * kp * 4};
  const cuuint32_t box[3] = {(cuuint32_t)kTBK, (cuuint32_t)box_rows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(SLAB_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return SLAB_OK;
}

size_t al256t(size_t b) { return (b + 255) / 256 * 256; }

template <int BN>
int launch_tf32s(cudaStream_t s, const CUtensorMap& tmA, const CUtensorMap& tmB, const TfArgs& a) {
  const size_t smem = tf32s_smem_bytes<BN>();
  SLAB_TRY(ensure_smem(tf32s_gemm_kernel<BN>, smem, "gemm_tf32s"));
  tf32s_gemm_kernel<BN><<<dim3(ceil_div(a.m, kTBM), ceil_div(a.n, BN), a.batch), 192, smem, s>>>(tmA, tmB, a);
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}

}  // namespace

// Slice arrays have their rows padded to whole tiles (128), so that no TMA box
// reaches past the array.
size_t gemm_tf32s_work_bytes(int m, int n, int k, int batch) {
  if (m <= 0 || n <= 0 || k <= 0 || batch <= 0) return 256;
  const size_t kp = (size_t)round_up(k, kTBK);
  const size_t mp = (size_t)round_up(m, kTBM), np_ = (size_t)round_up(n, kTBM);
  return al256t((size_t)kNSl * batch * mp * kp * 4) + al256t((size_t)kNSl * batch * np_ * kp * 4);
}

int gemm_tf32s(cudaStream_t s, int m, int n, int k, float alpha, const float* A, int lda, long long sA,
               const float* B, int ldb, long long sB, float beta, float* C, int ldc, long long sC, int batch,
               void* work, size_t work_bytes, int* err) {
  if (m <= 0 || n <= 0 || batch <= 0) return SLAB_OK;
  if (k <= 0 || !A || !B || !C || !work || !err || lda < m || ldb < k || ldc < m || batch > 65535)
    return set_error(SLAB_ERR_ARG, "gemm_tf32s: invalid arguments");
  if (work_bytes < gemm_tf32s_work_bytes(m, n, k, batch))
    return set_error(SLAB_ERR_ARG, "gemm_tf32s: work buffer too small");
  if (reinterpret_cast<uintptr_t>(work) % 256 != 0) return set_error(SLAB_ERR_ARG, "gemm_tf32s: work not aligned");
  const int kp = round_up(k, kTBK);
  const int mp = round_up(m, kTBM), np_ = round_up(n, kTBM);
  float* As = static_cast<float*>(work);
  float* Bs = reinterpret_cast<float*>(static_cast<unsigned char*>(work) + al256t((size_t)kNSl * batch * mp * kp * 4));
  split_a_kernel<<<dim3(mp / 32, kp / 32, batch), 256, 0, s>>>(A, lda, sA, m, mp, k, kp, batch, As);
  SLAB_CHECK_LAUNCH();
  const long long nb = (long long)np_ * kp;
  split_b_kernel<<<dim3((unsigned)((nb + 255) / 256), batch), 256, 0, s>>>(B, ldb, sB, n, np_, k, kp, batch, Bs);
  SLAB_CHECK_LAUNCH();
  const int BN = n <= 64 ? 64 : 128;
  CUtensorMap tmA, tmB;
  SLAB_TRY(make_f32_map(&tmA, As, kp, mp, kNSl * batch, kTBM));
  SLAB_TRY(make_f32_map(&tmB, Bs, kp, np_, kNSl * batch, BN));
  TfArgs ta{m, n, kp, batch, alpha, beta, C, ldc, sC, err};
  if (BN == 64) return launch_tf32s<64>(s, tmA, tmB, ta);
  return launch_tf32s<128>(s, tmA, tmB, ta);
}

}  // namespace slab

extern "C" size_t slab_sgemm_tc_work_bytes(int m, int n, int k, int batch) {
  return slab::gemm_tf32s_work_bytes(m, n, k, batch);
}

extern "C" int slab_sgemm_tc(int m, int n, int k, float alpha, const float* A, int lda, long long strideA,
                             const float* B, int ldb, long long strideB, float beta, float* C, int ldc,
                             long long strideC, int batch, void* work, size_t work_bytes, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the first 256 bytes of work hold the pipeline's error flag
  if (!work || work_bytes < 256 + slab::gemm_tf32s_work_bytes(m, n, k, batch))
    return slab::set_error(SLAB_ERR_ARG, "slab_sgemm_tc: work buffer too small");
  int* err = static_cast<int*>(work);
  SLAB_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
  SLAB_TRY(slab::gemm_tf32s(s, m, n, k, alpha, A, lda, strideA, B, ldb, strideB, beta, C, ldc, strideC, batch,
                            static_cast<unsigned char*>(work) + 256, work_bytes - 256, err));
  int h = 0;
  SLAB_CUDA_TRY(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  SLAB_CUDA_TRY(cudaStreamSynchronize(s));
  if (h != 0) return slab::set_error(SLAB_ERR_CUDA, "slab_sgemm_tc: tensor-core pipeline wait expired (code %d)", h);
  return SLAB_OK;
}
