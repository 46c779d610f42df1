// Shared definitions for the SlabLU GB300 kernels: status codes, error
// capture, small vector loads.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "../../include/slablu_gb300.h"

namespace slab {

// Record a message for slab_last_error(); returns the status passed in.
int set_error(int status, const char* fmt, ...);

#define SLAB_CUDA_TRY(expr)                                                        \
  do {                                                                             \
    cudaError_t e_ = (expr);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return ::slab::set_error(SLAB_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__,  \
                               #expr, cudaGetErrorString(e_));                     \
  } while (0)

// Every kernel launch of the library is followed by SLAB_CHECK_LAUNCH(), which
// also counts it (slab_launch_count()).
void count_launch();
#define SLAB_CHECK_LAUNCH()            \
  do {                                 \
    ::slab::count_launch();            \
    SLAB_CUDA_TRY(cudaGetLastError()); \
  } while (0)

#define SLAB_TRY(expr)                 \
  do {                                 \
    int s_ = (expr);                   \
    if (s_ != SLAB_OK) return s_;      \
  } while (0)

template <typename T>
struct vec4 {
  T x, y, z, w;
};

// 4 consecutive elements from shared memory; the address must be 4-element aligned.
__device__ __forceinline__ vec4<float> ld4(const float* p) {
  float4 v = *reinterpret_cast<const float4*>(p);
  return {v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ vec4<double> ld4(const double* p) {
  double2 a = *reinterpret_cast<const double2*>(p);
  double2 b = *reinterpret_cast<const double2*>(p + 2);
  return {a.x, a.y, b.x, b.y};
}

// Asynchronous copy of one 4- or 8-byte element from global to shared memory
// (cp.async, no register staging: a CTA can keep all of a tile's loads in
// flight).  Completed by cp_async_wait_all() followed by a block barrier.
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* sdst, const T* gsrc) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "cp.async element must be 4 or 8 bytes");
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(sdst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(sa), "l"(gsrc), "n"(sizeof(T)) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <typename T>
__device__ __forceinline__ T tabs(T v) {
  return v < T(0) ? -v : v;
}

__host__ __device__ inline int ceil_div(int a, int b) { return (a + b - 1) / b; }
__host__ __device__ inline int round_up(int a, int b) { return ceil_div(a, b) * b; }

}  // namespace slab
