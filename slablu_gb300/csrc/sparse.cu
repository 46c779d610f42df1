// Reduced sparse operator of the HPS discretisation on the device: the sum of
// the leaf DtN maps over the face unknowns (CSR), and its matrix-vector product.
// The CSR pattern is fixed by the leaf grid and is built once on the host
// (slablu_gb300/sparse.py); these kernels fill its values from the leaf DtN
// maps and apply it.
#include "common.cuh"

namespace slab {
namespace {

// vals[dest[i]] += src[i].  A reduced-operator entry collects the DtN entries of
// the one or two leaves that share its row's face, so at most two values meet
// in one slot and the sum does not depend on their order.
__global__ void csr_scatter_add_kernel(long long count, const double* __restrict__ src,
                                       const long long* __restrict__ dest, long long nnz, double* vals) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const long long d = dest[i];
    if (d >= 0 && d < nnz) atomicAdd(vals + d, src[i]);
  }
}

// y = alpha A x + beta y, one warp per row, lanes over the row's entries and a
// fixed-order shuffle reduction (deterministic).
__global__ void csr_spmv_kernel(int nrows, const long long* __restrict__ indptr, const int* __restrict__ indices,
                                const double* __restrict__ vals, const double* __restrict__ x, double alpha,
                                double beta, double* y) {
  const int lane = threadIdx.x & 31;
  const long long row = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  if (row >= nrows) return;
  double sum = 0.0;
  for (long long j = indptr[row] + lane; j < indptr[row + 1]; j += 32) sum += vals[j] * x[indices[j]];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) y[row] = (beta == 0.0 ? 0.0 : beta * y[row]) + alpha * sum;
}

}  // namespace
}  // namespace slab

extern "C" int slab_csr_assemble(long long count, const double* d_src, const long long* d_dest, long long nnz,
                                 double* d_vals, void* stream) {
  if (count < 0 || nnz < 0 || (count > 0 && (!d_src || !d_dest)) || (nnz > 0 && !d_vals))
    return slab::set_error(SLAB_ERR_ARG, "slab_csr_assemble: invalid arguments");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (nnz > 0) SLAB_CUDA_TRY(cudaMemsetAsync(d_vals, 0, (size_t)nnz * sizeof(double), s));
  if (count > 0) {
    const long long blocks = (count + 255) / 256;
    slab::csr_scatter_add_kernel<<<(unsigned)(blocks < 65535 * 8 ? blocks : 65535 * 8), 256, 0, s>>>(
        count, d_src, d_dest, nnz, d_vals);
    SLAB_CHECK_LAUNCH();
  }
  return SLAB_OK;
}

extern "C" int slab_csr_spmv(int nrows, const long long* d_indptr, const int* d_indices, const double* d_vals,
                             const double* d_x, double alpha, double beta, double* d_y, void* stream) {
  if (nrows < 0 || (nrows > 0 && (!d_indptr || !d_indices || !d_vals || !d_x || !d_y)))
    return slab::set_error(SLAB_ERR_ARG, "slab_csr_spmv: invalid arguments");
  if (nrows == 0) return SLAB_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long threads = (long long)nrows * 32;
  slab::csr_spmv_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(nrows, d_indptr, d_indices, d_vals, d_x,
                                                                         alpha, beta, d_y);
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}
