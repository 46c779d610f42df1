// FP32 matrix products on the tensor cores (tcgen05, kind::tf32) by exact
// three-way splitting of every operand into TF32 values (tcgemm.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace slab {

// Work bytes of gemm_tf32s for a batch of (m x k) (k x n) products.
size_t gemm_tf32s_work_bytes(int m, int n, int k, int batch);

// C[b] = alpha A[b] B[b] + beta C[b] for b < batch, column-major FP32 with
// uniform batch strides (sA, sB, sC elements).  Asynchronous on stream s.
// Each operand is split into three TF32 values whose sum is the FP32 value
// exactly; the six products of slice pairs with weights down to 2^-22 run on
// the tensor cores with FP32 accumulation in tensor memory; the error stays
// within the FP32 dot-product bound k 2^-24 max|A(i,:)| max|B(:,j)| (measured
// normwise 1.5e-6 at k = 200, a few times an FMA-chain FP32 product).  C may alias B (the operands are copied
// into `work` before the product runs).  err: device int, set nonzero if a
// pipeline wait expired (C is then not written).
int gemm_tf32s(cudaStream_t s, int m, int n, int k, float alpha, const float* A, int lda, long long sA,
               const float* B, int ldb, long long sB, float beta, float* C, int ldc, long long sC, int batch,
               void* work, size_t work_bytes, int* err);

}  // namespace slab
