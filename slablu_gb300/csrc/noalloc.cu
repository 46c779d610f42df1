// Allocation-free variant of the batched leaf DtN entry point.
//
// Some callers cannot allocate device memory at the point where they need
// leaf DtN maps: host applications whose device memory is owned by their own
// pool allocator and that forbid allocations by libraries, or programs that fix
// their device-memory budget at start-up, where an allocation inside a library
// call would fail or break that budget.
// slab_leaf_dtn needs a work area for the leaf LU factors; this variant uses
// a fixed scratch array compiled into the library instead, so the caller only
// provides inputs and outputs.
//
// The scratch is one file-scope __device__ array of SLAB_NOALLOC_SCRATCH_BYTES
// bytes; every GPU that loads the library holds it until the process exits.
// All calls share it: the last call's contents stay there, and calls whose
// kernels overlap on the GPU (different streams, or other host threads) race
// on it.  Nothing in it has to start at zero: every element the kernels read
// was written earlier in the same call.
#include <mutex>

#include "leaf.cuh"

#define SLAB_NOALLOC_SCRATCH_BYTES (64ull << 20)

namespace slab {

int leaf_dtn_with_work(int nleaf, int p, const LeafCoeffs& co, const double* D, const double* Dsq, const double* Nx,
                       int precision, void* work, size_t work_bytes, double* dtn_out, double* S_out, int* info,
                       cudaStream_t s);

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[SLAB_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  The host-side
// symbol is only a stand-in and must never be passed to a kernel; the address
// is looked up once per device, with that device current.
int scratch_address(void** out) {
  int dev = 0;
  SLAB_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return set_error(SLAB_ERR_ARG, "slab_leaf_dtn_noalloc: device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return set_error(SLAB_ERR_CUDA, "slab_leaf_dtn_noalloc: cudaGetSymbolAddress failed: %s",
                       cudaGetErrorString(e));
    g_scratch_addr[dev] = ptr;
  }
  *out = g_scratch_addr[dev];
  return SLAB_OK;
}

}  // namespace
}  // namespace slab

extern "C" size_t slab_leaf_dtn_noalloc_max_bytes(void) { return SLAB_NOALLOC_SCRATCH_BYTES; }

extern "C" int slab_leaf_dtn_noalloc(int nleaf, int p, const double* c11, const double* c22, const double* c1,
                                     const double* c2, const double* c, const double* D, const double* Dsq,
                                     const double* Nx, int precision, double* dtn, int* info, void* stream) {
  if (nleaf <= 0 || p < 4 || !D || !Dsq || !Nx || !dtn)
    return slab::set_error(SLAB_ERR_ARG, "slab_leaf_dtn_noalloc: invalid argument");
  if (precision != SLAB_PREC_FP64 && precision != SLAB_PREC_FP32 && precision != SLAB_PREC_MIXED)
    return slab::set_error(SLAB_ERR_ARG, "slab_leaf_dtn_noalloc: unknown precision %d", precision);
  const size_t need = slab_leaf_dtn_work_bytes(nleaf, p, precision);
  if (need > SLAB_NOALLOC_SCRATCH_BYTES)
    return slab::set_error(SLAB_ERR_ARG,
                           "slab_leaf_dtn_noalloc: %d leaves of order p=%d need %zu bytes of scratch, more than the "
                           "built-in %llu bytes; split the batch or use slab_leaf_dtn with a work buffer",
                           nleaf, p, need, (unsigned long long)SLAB_NOALLOC_SCRATCH_BYTES);
  void* scratch = nullptr;
  const int st = slab::scratch_address(&scratch);
  if (st != SLAB_OK) return st;
  // the c12-free leaf path only: its work size is slab_leaf_dtn_work_bytes (the
  // mixed-derivative variant needs slab_leaf_dtn_mixed_work_bytes and is not
  // offered here)
  slab::LeafCoeffs co{c11, c22, c1, c2, c};
  return slab::leaf_dtn_with_work(nleaf, p, co, D, Dsq, Nx, precision, scratch, need, dtn, nullptr, info,
                                  static_cast<cudaStream_t>(stream));
}
