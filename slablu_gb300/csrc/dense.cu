// Host launchers for the dense building blocks (float and double).
#include <atomic>
#include <cstdarg>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <type_traits>

#include "dense.cuh"

namespace slab {

namespace {
thread_local std::string g_last_error;
std::atomic<long long> g_launches{0};
}

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }
void add_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int set_error(int status, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return status;
}

const char* last_error() { return g_last_error.c_str(); }

size_t smem_limit_bytes() {
  static size_t v = 0;
  if (v == 0) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    v = optin > 0 ? (size_t)optin : 48 * 1024;
  }
  return v;
}

size_t allow_dynamic_smem(const void* kernel) {
  static std::mutex mu;
  static std::map<const void*, size_t> done;
  std::lock_guard<std::mutex> lock(mu);
  auto it = done.find(kernel);
  if (it != done.end()) return it->second;
  cudaFuncAttributes fa{};
  if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  const size_t lim = smem_limit_bytes() > fa.sharedSizeBytes ? smem_limit_bytes() - fa.sharedSizeBytes : 0;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lim) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  done[kernel] = lim;
  return lim;
}

__global__ void perm_from_ipiv_kernel(const int* ipiv, int n, int* perm) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int i = 0; i < n; ++i) perm[i] = i;
  for (int j = 0; j < n; ++j) {
    const int pj = ipiv[j];
    if (pj != j && pj >= 0 && pj < n) {
      const int t = perm[j];
      perm[j] = perm[pj];
      perm[pj] = t;
    }
  }
}

__global__ void perm_batched_kernel(const int* ipiv, long long strideP, int n, int batch, int* perm,
                                    long long strideQ) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  const int* iv = ipiv + strideP * b;
  int* pm = perm + strideQ * b;
  for (int i = 0; i < n; ++i) pm[i] = i;
  for (int j = 0; j < n; ++j) {
    const int pj = iv[j];
    if (pj != j && pj >= 0 && pj < n) {
      const int t = pm[j];
      pm[j] = pm[pj];
      pm[pj] = t;
    }
  }
}

int build_perm_batched(cudaStream_t s, const int* ipiv, long long strideP, int n, int batch, int* perm,
                       long long strideQ) {
  if (batch <= 0) return SLAB_OK;
  perm_batched_kernel<<<ceil_div(batch, 128), 128, 0, s>>>(ipiv, strideP, n, batch, perm, strideQ);
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}

static int sm_count();

template <typename T>
int getrs_small(cudaStream_t s, int n, int nrhs, const T* LU, const long long* offLU, long long strideLU, int lda,
                const int* perm, const long long* offP, long long strideP, T* B, const long long* offB,
                long long strideB, int ldb, int batch) {
  if (n <= 0 || nrhs <= 0 || batch <= 0) return SLAB_OK;
  if (nrhs > 4) return set_error(SLAB_ERR_ARG, "getrs_small: nrhs %d > 4", nrhs);
  if (n > 32 * kWarpSlots) return set_error(SLAB_ERR_ARG, "getrs_small: order %d > %d", n, 32 * kWarpSlots);
  // few large matrices (the top merge levels): one CTA per matrix instead of one warp
  const bool per_cta = n >= 128 && batch <= 4 * sm_count();
  const size_t bytes = (size_t)(per_cta ? 1 : kWarpSolveWarps) * n * nrhs * sizeof(T);
  auto launch = [&](auto kern) -> int {
    SLAB_TRY(ensure_smem(kern, bytes, "getrs_small"));
    if (per_cta)
      kern<<<batch, 256, bytes, s>>>(n, LU, offLU, strideLU, lda, perm, offP, strideP, B, offB, strideB, ldb, batch);
    else
      kern<<<ceil_div(batch, kWarpSolveWarps), 32 * kWarpSolveWarps, bytes, s>>>(n, LU, offLU, strideLU, lda, perm,
                                                                                 offP, strideP, B, offB, strideB, ldb,
                                                                                 batch);
    return SLAB_OK;
  };
  switch (nrhs) {
    case 1: SLAB_TRY(per_cta ? launch(getrs_cta_blocked_kernel<T, 1>) : launch(getrs_warp_blocked_kernel<T, 1>)); break;
    case 2: SLAB_TRY(per_cta ? launch(getrs_cta_blocked_kernel<T, 2>) : launch(getrs_warp_blocked_kernel<T, 2>)); break;
    case 3: SLAB_TRY(per_cta ? launch(getrs_cta_blocked_kernel<T, 3>) : launch(getrs_warp_blocked_kernel<T, 3>)); break;
    default:
      SLAB_TRY(per_cta ? launch(getrs_cta_blocked_kernel<T, 4>) : launch(getrs_warp_blocked_kernel<T, 4>));
      break;
  }
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}

template <typename T>
int getrs_many(cudaStream_t s, int n, int nrhs, const T* LU, long long strideLU, int lda, const int* perm,
               long long strideP, T* B, long long strideB, int ldb, int batch) {
  if (n <= 0 || nrhs <= 0 || batch <= 0) return SLAB_OK;
  const size_t bytes = getrs_many_smem_bytes(n, sizeof(T));
  SLAB_TRY(ensure_smem(getrs_many_kernel<T>, bytes, "getrs_many"));
  const int tiles = ceil_div(nrhs, kManyCols);
  if (tiles > 65535) return set_error(SLAB_ERR_ARG, "getrs_many: %d right-hand sides is too many", nrhs);
  dim3 grid(batch, tiles);
  getrs_many_kernel<T><<<grid, 256, bytes, s>>>(n, nrhs, LU, strideLU, lda, perm, strideP, B, strideB, ldb);
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}
template <typename T>
bool getrs_many_fits(int n) {
  return n <= kManyMaxN &&
         getrs_many_smem_bytes(n, sizeof(T)) <= allow_dynamic_smem(reinterpret_cast<const void*>(getrs_many_kernel<T>));
}
template bool getrs_many_fits<float>(int);
template bool getrs_many_fits<double>(int);
template int getrs_many<float>(cudaStream_t, int, int, const float*, long long, int, const int*, long long, float*,
                               long long, int, int);
template int getrs_many<double>(cudaStream_t, int, int, const double*, long long, int, const int*, long long,
                                double*, long long, int, int);

template <typename T>
int trsv_coop(cudaStream_t s, const T* LU, int lda, int n, const int* perm, const T* Linv, const T* Uinv, int bs,
              const T* B, int ldb, T* X, int ldx, int nrhs, bool trans) {
  if (n <= 0 || nrhs <= 0) return SLAB_OK;
  if (nrhs > kCoopMaxRhs) return set_error(SLAB_ERR_ARG, "trsv_coop: nrhs %d > %d", nrhs, kCoopMaxRhs);
  const size_t bytes = ((size_t)kCoopMaxOwn * bs * nrhs + (size_t)bs * (bs + 1) + (size_t)bs * nrhs) * sizeof(T);
  SLAB_TRY(ensure_smem(trsv_coop_kernel<T>, bytes, "trsv_coop"));
  int dev = 0, sms = 0, per_sm = 0;
  SLAB_CUDA_TRY(cudaGetDevice(&dev));
  SLAB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  SLAB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trsv_coop_kernel<T>, 256, bytes));
  const int max_grid = sms * (per_sm > 0 ? per_sm : 0);
  const int nblk = ceil_div(n, bs);
  const int G = nblk < max_grid ? nblk : max_grid;
  if (G <= 0 || ceil_div(nblk, G) > kCoopMaxOwn)
    return set_error(SLAB_ERR_ARG, "trsv_coop: order %d too large for a co-resident grid", n);
  int tr = trans ? 1 : 0;
  void* args[] = {(void*)&LU, (void*)&lda, (void*)&n, (void*)&perm, (void*)&Linv, (void*)&Uinv, (void*)&bs,
                  (void*)&B, (void*)&ldb, (void*)&X, (void*)&ldx, (void*)&nrhs, (void*)&tr};
  SLAB_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)trsv_coop_kernel<T>, dim3(G), dim3(256), args, bytes, s));
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}

namespace {
// Largest usable cluster (16 when the device allows non-portable cluster sizes
// for this kernel at this shared-memory footprint and block size, else 8).
int cluster_size_for(const void* kernel, size_t bytes, int threads) {
  static std::mutex mu;
  static std::map<std::tuple<const void*, int, size_t, int>, int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 8;
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_tuple(kernel, dev, bytes, threads);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  int best = 8;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(16);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = bytes;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 16;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nc = 0;
    if (cudaOccupancyMaxActiveClusters(&nc, kernel, &cfg) == cudaSuccess && nc > 0) best = 16;
  }
  cudaGetLastError();  // a refused query leaves no error behind
  cache[key] = best;
  return best;
}

int launch_cluster(const void* kernel, int cl, int threads, size_t bytes, cudaStream_t s, void** args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cl);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = bytes;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = cl;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  SLAB_CUDA_TRY(cudaLaunchKernelExC(&cfg, kernel, args));
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}
}  // namespace

template <typename T>
int trsv_cluster(cudaStream_t s, const T* LU, int lda, int n, const int* perm, const T* Linv, const T* Uinv,
                 const T* B, int ldb, T* X, int ldx, int nrhs, bool trans) {
  if (n <= 0 || nrhs <= 0) return SLAB_OK;
  if (nrhs > kCoopMaxRhs) return set_error(SLAB_ERR_ARG, "trsv_cluster: nrhs %d > %d", nrhs, kCoopMaxRhs);
  const int nblk = ceil_div(n, kClBs);
  const size_t lim = allow_dynamic_smem(reinterpret_cast<const void*>(trsv_cluster_kernel<T>));
  auto bytes_for = [&](int cl) {
    const int own = ceil_div(nblk, cl);
    return (size_t)(5 * own + 3) * kClBs * kCoopMaxRhs * sizeof(T);
  };
  const void* kern = reinterpret_cast<const void*>(trsv_cluster_kernel<T>);
  int CL = cluster_size_for(kern, bytes_for(16), 256);
  if (CL > nblk) CL = nblk < 8 ? nblk : 8;
  int own_max = ceil_div(nblk, CL);
  const size_t bytes = bytes_for(CL);
  if (bytes > lim) return set_error(SLAB_ERR_ARG, "trsv_cluster: order %d too large", n);
  int tr = trans ? 1 : 0;
  void* args[] = {(void*)&LU, (void*)&lda, (void*)&n, (void*)&perm, (void*)&Linv, (void*)&Uinv, (void*)&B,
                  (void*)&ldb, (void*)&X, (void*)&ldx, (void*)&nrhs, (void*)&tr, (void*)&own_max};
  return launch_cluster(kern, CL, 256, bytes, s, args);
}

template <typename T>
int getrs_small_t(cudaStream_t s, int n, int nrhs, const T* LU, const long long* offLU, long long strideLU, int lda,
                  const int* perm, const long long* offP, long long strideP, T* B, const long long* offB,
                  long long strideB, int ldb, int batch) {
  if (n <= 0 || nrhs <= 0 || batch <= 0) return SLAB_OK;
  if (nrhs > 4) return set_error(SLAB_ERR_ARG, "getrs_small_t: nrhs %d > 4", nrhs);
  if (n > 32 * kWarpSlots) return set_error(SLAB_ERR_ARG, "getrs_small_t: order %d > %d", n, 32 * kWarpSlots);
  const size_t bytes = (size_t)kWarpSolveWarps * n * nrhs * sizeof(T);
  SLAB_TRY(ensure_smem(getrs_warp_t_kernel<T>, bytes, "getrs_small_t"));
  getrs_warp_t_kernel<T><<<ceil_div(batch, kWarpSolveWarps), 32 * kWarpSolveWarps, bytes, s>>>(
      n, nrhs, LU, offLU, strideLU, lda, perm, offP, strideP, B, offB, strideB, ldb, batch);
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}

template <typename T>
int gemm_tn(cudaStream_t s, int m, int n, int k, T alpha, const T* A, const long long* offA, long long strideA,
            int lda, const T* B, const long long* offB, long long strideB, int ldb, T beta, T* C,
            const long long* offC, long long strideC, int ldc, int batch) {
  if (m <= 0 || n <= 0 || batch <= 0) return SLAB_OK;
  if (batch > 65535) {
    for (int b0 = 0; b0 < batch; b0 += 65535) {
      const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
      SLAB_TRY(gemm_tn<T>(s, m, n, k, alpha, offA ? A : A + strideA * b0, offA ? offA + b0 : nullptr, strideA, lda,
                          offB ? B : B + strideB * b0, offB ? offB + b0 : nullptr, strideB, ldb, beta,
                          offC ? C : C + strideC * b0, offC ? offC + b0 : nullptr, strideC, ldc, nb));
    }
    return SLAB_OK;
  }
  const int kk = k < 0 ? 0 : k;
  if (n <= 16) {
    dim3 g(ceil_div(m, 8), 1, batch);
#define SLAB_TN(NC)                                                                                           \
  gemm_tn_narrow_kernel<T, NC><<<g, 256, 0, s>>>(m, n, kk, alpha, A, offA, strideA, lda, B, offB, strideB, ldb, \
                                                 beta, C, offC, strideC, ldc)
    if (n <= 1)
      SLAB_TN(1);
    else if (n <= 2)
      SLAB_TN(2);
    else if (n <= 4)
      SLAB_TN(4);
    else if (n <= 8)
      SLAB_TN(8);
    else
      SLAB_TN(16);
#undef SLAB_TN
    SLAB_CHECK_LAUNCH();
    return SLAB_OK;
  }
  dim3 grid(ceil_div(m, 64), ceil_div(n, 64), batch);
  gemm_kernel<T, true><<<grid, 256, 0, s>>>(m, n, kk, alpha, A, offA, strideA, lda, B, offB, strideB, ldb, beta, C,
                                           offC, strideC, ldc);
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}

// The same with the permutation and the pivots in shared memory (2 n ints): the
// sequential interchanges cost shared-memory latencies instead of global ones.
__global__ void perm_from_ipiv_smem_kernel(const int* ipiv, int n, int* perm) {
  extern __shared__ int psm[];
  int* p = psm;
  int* iv = psm + n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    p[i] = i;
    iv[i] = ipiv[i];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int j = 0; j < n; ++j) {
      const int pj = iv[j];
      if (pj != j && pj >= 0 && pj < n) {
        const int t = p[j];
        p[j] = p[pj];
        p[pj] = t;
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = p[i];
}

int build_perm(cudaStream_t s, const int* ipiv, int n, int* perm) {
  const size_t bytes = 2 * (size_t)n * sizeof(int);
  if (bytes <= 48 * 1024) {
    perm_from_ipiv_smem_kernel<<<1, 256, bytes, s>>>(ipiv, n, perm);
  } else {
    perm_from_ipiv_kernel<<<1, 1, 0, s>>>(ipiv, n, perm);
  }
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}

// Multiprocessor count of the current device (queried once per device).
static int sm_count() {
  static std::mutex mu;
  static std::map<int, int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return 152;
  }
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(dev);
  if (it != cache.end()) return it->second;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
    cudaGetLastError();
    sms = 152;
  }
  cache[dev] = sms;
  return sms;
}

// Tile policy of the FP32 products issued by this host thread: 0 = 128 x 128 tiles
// where their grid fills the GPU, 1 = always 64 x 64 (an engine sets it from its
// SLAB_OPT_GEMM_TILES around its work, so graphs capture the policy they ran with;
// SLAB_GEMM64=1 forces 1 for comparisons).
static thread_local int g_gemm_tiles = 0;
void set_gemm_tiles(int policy) { g_gemm_tiles = policy; }
static bool gemm64_only() {
  if (g_gemm_tiles == 1) return true;
  const char* e = getenv("SLAB_GEMM64");
  return e && e[0] == '1';
}

// FP32 product C = beta*C + alpha * A B (column-major, batched like gemm_kernel)
// with 128 x 128 output tiles: 256 threads, 8 x 8 outputs per thread (two 4-row
// by two 4-column groups, so each k step reads four float4 from shared memory
// for 64 FMAs), k staged 8 at a time in double-buffered shared memory; the next
// k slice is loaded into registers while the current one is multiplied, so one
// __syncthreads per slice.  For products whose 128-wide tiles fill the GPU.
constexpr int kG8K = 8;
constexpr int kG8LD = 132;  // 128 + 4: the float4 reads stay 16-byte aligned
__global__ void __launch_bounds__(256) gemm128_kernel(int m, int n, int k, float alpha, const float* __restrict__ A,
                                                     const long long* offA, long long strideA, int lda,
                                                     const float* __restrict__ B, const long long* offB,
                                                     long long strideB, int ldb, float beta, float* C,
                                                     const long long* offC, long long strideC, int ldc) {
  __shared__ __align__(16) float As[2][kG8K * kG8LD];
  __shared__ __align__(16) float Bs[2][kG8K * kG8LD];
  const int bz = blockIdx.z;
  A += batch_off(offA, strideA, bz);
  B += batch_off(offB, strideB, bz);
  C += batch_off(offC, strideC, bz);
  const int r0 = blockIdx.x * 128, c0 = blockIdx.y * 128;
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  // loads: A slice 128 x 8 (thread: rows ar + 32 q, column ak), B slice 8 x 128 (thread: row bk, columns bc + 32 q)
  const int ar = tid & 31, ak = tid >> 5;
  const int bk = tid & 7, bc = tid >> 3;
  float ra[4], rb[4];
  auto load = [&](int k0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int gr = r0 + ar + 32 * q, gk = k0 + ak;
      ra[q] = (gr < m && gk < k) ? A[gr + (size_t)gk * lda] : 0.f;
      const int gc = c0 + bc + 32 * q, gk2 = k0 + bk;
      rb[q] = (gc < n && gk2 < k) ? B[gk2 + (size_t)gc * ldb] : 0.f;
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      As[buf][(ar + 32 * q) + ak * kG8LD] = ra[q];
      Bs[buf][(bc + 32 * q) + bk * kG8LD] = rb[q];
    }
  };
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
  const int nk = (k + kG8K - 1) / kG8K;
  if (nk > 0) {
    load(0);
    store(0);
  }
  __syncthreads();
  for (int t = 0; t < nk; ++t) {
    const int buf = t & 1;
    if (t + 1 < nk) load((t + 1) * kG8K);
    const float* as = As[buf];
    const float* bs = Bs[buf];
#pragma unroll
    for (int kk = 0; kk < kG8K; ++kk) {
      const float4 a0 = *reinterpret_cast<const float4*>(as + 4 * tx + kk * kG8LD);
      const float4 a1 = *reinterpret_cast<const float4*>(as + 64 + 4 * tx + kk * kG8LD);
      const float4 b0 = *reinterpret_cast<const float4*>(bs + 4 * ty + kk * kG8LD);
      const float4 b1 = *reinterpret_cast<const float4*>(bs + 64 + 4 * ty + kk * kG8LD);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] += a[i] * b[j];
    }
    if (t + 1 < nk) store(buf ^ 1);
    __syncthreads();
  }
  // rows 4 tx + {0..3} and 64 + 4 tx + {0..3}; columns 4 ty + {0..3} and 64 + 4 ty + {0..3}
#pragma unroll
  for (int jb = 0; jb < 2; ++jb) {
    float cv[4][8];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = c0 + 64 * jb + 4 * ty + j;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int r = r0 + (i < 4 ? 4 * tx + i : 64 + 4 * tx + i - 4);
        cv[j][i] = (beta != 0.f && c < n && r < m) ? C[r + (size_t)c * ldc] : 0.f;
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = c0 + 64 * jb + 4 * ty + j;
      if (c >= n) continue;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int r = r0 + (i < 4 ? 4 * tx + i : 64 + 4 * tx + i - 4);
        if (r < m) C[r + (size_t)c * ldc] = (beta == 0.f ? 0.f : beta * cv[j][i]) + alpha * acc[i][4 * jb + j];
      }
    }
  }
}

template <typename T>
int gemm(cudaStream_t s, int m, int n, int k, T alpha, const T* A, const long long* offA, long long strideA,
         int lda, const T* B, const long long* offB, long long strideB, int ldb, T beta, T* C,
         const long long* offC, long long strideC, int ldc, int batch) {
  if (m <= 0 || n <= 0 || batch <= 0) return SLAB_OK;
  if (batch > 1 && !offA && !offB && !offC && strideA == 0 && strideB == (long long)ldb * n &&
      strideC == (long long)ldc * n && (long long)n * batch <= 65535LL * 64) {
    // one A for every entry and the B and C blocks back to back: a single product
    // of n * batch columns (the leaves' flux products of a solve)
    return gemm<T>(s, m, n * batch, k, alpha, A, nullptr, 0, lda, B, nullptr, 0, ldb, beta, C, nullptr, 0, ldc, 1);
  }
  if (batch > 65535) {
    // grid.z limit: split the batch (offset arrays or strides advance per chunk)
    for (int b0 = 0; b0 < batch; b0 += 65535) {
      const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
      SLAB_TRY(gemm<T>(s, m, n, k, alpha, offA ? A : A + strideA * b0, offA ? offA + b0 : nullptr, strideA, lda,
                       offB ? B : B + strideB * b0, offB ? offB + b0 : nullptr, strideB, ldb, beta,
                       offC ? C : C + strideC * b0, offC ? offC + b0 : nullptr, strideC, ldc, nb));
    }
    return SLAB_OK;
  }
  if (n <= 16 && batch == 1 && !offA && !offB && !offC && k >= 512 && ceil_div(m, 256) < 64) {
    // tall-skinny single product: split k over CTAs, accumulate with atomics
    // (chunks of 64: a 2000 x 2000 matrix-vector product spreads over 256 CTAs)
    const int mb = ceil_div(m, 256);
    int nsplit = ceil_div(256, mb);
    const int kchunk = 64;
    nsplit = nsplit < ceil_div(k, kchunk) ? nsplit : ceil_div(k, kchunk);
    if (beta != T(1)) {
      scale_kernel<T><<<ceil_div(m * n, 256), 256, 0, s>>>(C, m, n, ldc, beta);
      SLAB_CHECK_LAUNCH();
    }
    for (int ks = 0; ks < k; ks += kchunk * nsplit) {
      const int kk = k - ks < kchunk * nsplit ? k - ks : kchunk * nsplit;
      dim3 g(mb, ceil_div(kk, kchunk));
#define SLAB_SPLIT(NC)                                                                                             \
  gemm_narrow_splitk_kernel<T, NC><<<g, 256, 0, s>>>(m, n, kk, kchunk, alpha, A + (size_t)ks * lda, lda, B + ks, ldb, \
                                                     C, ldc)
      if (n <= 1)
        SLAB_SPLIT(1);
      else if (n <= 2)
        SLAB_SPLIT(2);
      else if (n <= 4)
        SLAB_SPLIT(4);
      else if (n <= 8)
        SLAB_SPLIT(8);
      else
        SLAB_SPLIT(16);
#undef SLAB_SPLIT
      SLAB_CHECK_LAUNCH();
    }
    return SLAB_OK;
  }
  if (n <= 16) {
    dim3 g(ceil_div(m, 256), 1, batch);
    const int kk = k < 0 ? 0 : k;
    // a grid of few CTAs with long rows (the top merge levels: ten slabs, thousands of
    // columns): split k over the warps of a CTA, 32 rows per CTA
    const bool ks = (long long)ceil_div(m, 256) * batch < 2LL * sm_count() && kk >= 128;
    if (ks) g = dim3(ceil_div(m, 32), 1, batch);
#define SLAB_NARROW(NC)                                                                                        \
  do {                                                                                                         \
    if (ks)                                                                                                    \
      gemm_narrow_ks_kernel<T, NC><<<g, 256, 0, s>>>(m, n, kk, alpha, A, offA, strideA, lda, B, offB, strideB, \
                                                     ldb, beta, C, offC, strideC, ldc);                       \
    else                                                                                                       \
      gemm_narrow_kernel<T, NC><<<g, 256, 0, s>>>(m, n, kk, alpha, A, offA, strideA, lda, B, offB, strideB,    \
                                                  ldb, beta, C, offC, strideC, ldc);                          \
  } while (0)
    if (n <= 1)
      SLAB_NARROW(1);
    else if (n <= 2)
      SLAB_NARROW(2);
    else if (n <= 4)
      SLAB_NARROW(4);
    else if (n <= 8)
      SLAB_NARROW(8);
    else
      SLAB_NARROW(16);
#undef SLAB_NARROW
    SLAB_CHECK_LAUNCH();
    return SLAB_OK;
  }
  // k == 0 leaves the k loop empty: C = beta*C
  if (std::is_same<T, double>::value && (long long)ceil_div(m, 64) * ceil_div(n, 64) * batch < 2LL * sm_count()) {
    dim3 g32(ceil_div(m, 32), ceil_div(n, 32), batch);
    gemm32_kernel<T><<<g32, 256, 0, s>>>(m, n, k < 0 ? 0 : k, alpha, A, offA, strideA, lda, B, offB, strideB, ldb,
                                         beta, C, offC, strideC, ldc);
    SLAB_CHECK_LAUNCH();
    return SLAB_OK;
  }
  if constexpr (std::is_same<T, float>::value) {
    // 128-wide tiles only where they still give every SM a CTA (narrow products,
    // e.g. one 256-column outer block, keep the 64 x 64 grid and its parallelism)
    if (m >= 128 && n >= 128 && !gemm64_only() &&
        (long long)ceil_div(m, 128) * ceil_div(n, 128) * batch >= sm_count()) {
      dim3 g128(ceil_div(m, 128), ceil_div(n, 128), batch);
      gemm128_kernel<<<g128, 256, 0, s>>>(m, n, k < 0 ? 0 : k, alpha, A, offA, strideA, lda, B, offB, strideB, ldb,
                                          beta, C, offC, strideC, ldc);
      SLAB_CHECK_LAUNCH();
      return SLAB_OK;
    }
  }
  dim3 grid(ceil_div(m, 64), ceil_div(n, 64), batch);
  gemm_kernel<T, false><<<grid, 256, 0, s>>>(m, n, k < 0 ? 0 : k, alpha, A, offA, strideA, lda, B, offB, strideB, ldb,
                                      beta, C, offC, strideC, ldc);
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}

template <typename T>
int getrf_batched(cudaStream_t s, int n, int nc, T* A, const long long* offA, long long strideA, int lda,
                  int* piv, const long long* offP, long long strideP, int* info, int batch) {
  if (n <= 0 || batch <= 0) return SLAB_OK;
  const size_t bytes = (size_t)getrf_smem_elems(n) * sizeof(T);
  SLAB_TRY(ensure_smem(getrf_batched_kernel<T>, bytes, "getrf_batched"));
  getrf_batched_kernel<T><<<batch, kNT, bytes, s>>>(n, nc, A, offA, strideA, lda, piv, offP, strideP, info);
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}

template <typename T>
int getrs_batched(cudaStream_t s, int n, int nrhs, const T* LU, const long long* offLU, long long strideLU,
                  int lda, const int* piv, const long long* offP, long long strideP, T* B,
                  const long long* offB, long long strideB, int ldb, int batch, bool lower, bool upper) {
  if (n <= 0 || nrhs <= 0 || batch <= 0) return SLAB_OK;
  const size_t limit = allow_dynamic_smem(reinterpret_cast<const void*>(getrs_batched_kernel<T>));
  int tile = getrs_tile_cols(n, sizeof(T), limit);
  if (tile > round_up(nrhs, 4)) tile = round_up(nrhs, 4);  // do not reserve unused columns
  if (tile <= 0) return set_error(SLAB_ERR_ARG, "getrs_batched: order %d too large for shared memory", n);
  const size_t bytes = (size_t)getrs_smem_elems(n, tile) * sizeof(T);
  SLAB_TRY(ensure_smem(getrs_batched_kernel<T>, bytes, "getrs_batched"));
  const int ntiles = ceil_div(nrhs, tile);
  if (ntiles > 65535) return set_error(SLAB_ERR_ARG, "getrs_batched: %d right-hand sides is too many", nrhs);
  dim3 grid(batch, ntiles);
  getrs_batched_kernel<T><<<grid, kNT, bytes, s>>>(n, nrhs, tile, LU, offLU, strideLU, lda, piv, offP, strideP, B,
                                                  offB, strideB, ldb, lower ? 1 : 0, upper ? 1 : 0);
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}

// Pivoted FP32 panel (rows k0..n, columns k0..k0+nb, nb <= 32) in ONE CTA of NT
// threads, for m = n - k0 <= 4 NT: thread t owns the physical rows t and t + NT
// in registers and t + 2NT, t + 3NT in shared memory (column-major, ld 2NT).
// The register rows are kept rotated -- entry k holds column j + k at step j, so
// the current column is entry 0 and every register index is static -- and turn
// once per step; the j loop is unrolled by four so that the compiler renames
// three of the four turns away.  One __syncthreads per column: the owner of
// each warp's best candidate (magnitude key, then the smaller logical index)
// publishes the candidate row, rotated and zero-padded, in a double-buffered
// slot; after the barrier every warp reduces the slots itself, relabels the
// interchange, forms its multipliers and updates its rows (register rows with
// all 31 FMAs against the zero padding, shared-memory rows with exactly the
// 31 - j columns left).  A slot buffer is rewritten two columns later, after a
// barrier that every reader of it has passed.  The pivot sequence is LAPACK's,
// and each entry sees the same operations in the same order as in
// biglu_panel_cluster_kernel, so both give the same factors.  At the end each
// thread writes its rows to their logical positions, and L11^{-1} goes to linv.
// above this height the cluster kernel is faster
constexpr int kPanelCtaMaxRows = 1536;
template <int NT>
__host__ __device__ inline size_t panel_cta_smem_bytes() {
  constexpr int NW = NT / 32;
  return ((size_t)2 * NT * kNB + 2 * NW * kNB + 2 * (size_t)kNB * (kNB + 1)) * sizeof(float) +
         2 * NW * (sizeof(unsigned) + sizeof(int));
}

// x[c * LDS] -= l * p[c - j] for c = j+1 .. 31, exactly the columns left (x:
// column 0 of a shared-memory row; p: the rotated pivot row)
template <int LDS>
__device__ __forceinline__ void smem_row_update(float* x, int j, float l, const float* p) {
  float* y = x + j * LDS;
  switch (31 - j) {
#define SLAB_PANEL_UPD(K) \
  case K:                 \
    y[K * LDS] -= l * p[K];
    SLAB_PANEL_UPD(31) SLAB_PANEL_UPD(30) SLAB_PANEL_UPD(29) SLAB_PANEL_UPD(28) SLAB_PANEL_UPD(27)
    SLAB_PANEL_UPD(26) SLAB_PANEL_UPD(25) SLAB_PANEL_UPD(24) SLAB_PANEL_UPD(23) SLAB_PANEL_UPD(22)
    SLAB_PANEL_UPD(21) SLAB_PANEL_UPD(20) SLAB_PANEL_UPD(19) SLAB_PANEL_UPD(18) SLAB_PANEL_UPD(17)
    SLAB_PANEL_UPD(16) SLAB_PANEL_UPD(15) SLAB_PANEL_UPD(14) SLAB_PANEL_UPD(13) SLAB_PANEL_UPD(12)
    SLAB_PANEL_UPD(11) SLAB_PANEL_UPD(10) SLAB_PANEL_UPD(9) SLAB_PANEL_UPD(8) SLAB_PANEL_UPD(7)
    SLAB_PANEL_UPD(6) SLAB_PANEL_UPD(5) SLAB_PANEL_UPD(4) SLAB_PANEL_UPD(3) SLAB_PANEL_UPD(2)
    SLAB_PANEL_UPD(1)
#undef SLAB_PANEL_UPD
    default:
      break;
  }
}

template <int NT>
__global__ void __launch_bounds__(NT, 1)
    biglu_panel_cta_kernel(float* A, int lda, int n, int k0, int nb, int* ipiv, int* info, float* linv, int* gath) {
  constexpr int NW = NT / 32, LDS = 2 * NT, W = kNB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* S = reinterpret_cast<float*>(smem_raw);  // LDS x W: physical rows 2NT .. 4NT-1
  float* srow = S + (size_t)LDS * W;             // [2][NW][W]: pivot candidates, rotated (entry k = column j + k)
  float* Ls = srow + 2 * NW * W;
  float* Xs = Ls + W * (W + 1);
  unsigned* skey = reinterpret_cast<unsigned*>(Xs + W * (W + 1));
  int* sli = reinterpret_cast<int*>(skey + 2 * NW);
  const int m = n - k0;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float r0[W], r1[W];
  int li0 = tid < m ? tid : INT_MAX, li1 = tid + NT < m ? tid + NT : INT_MAX;
  int li2 = tid + 2 * NT < m ? tid + 2 * NT : INT_MAX, li3 = tid + 3 * NT < m ? tid + 3 * NT : INT_MAX;
  float* s2 = S + tid;
  float* s3 = S + tid + NT;
#pragma unroll
  for (int c = 0; c < W; ++c) {
    const float* col = A + (size_t)(k0 + c) * lda + k0;
    const bool cv = c < nb;
    r0[c] = cv && li0 != INT_MAX ? col[tid] : 0.f;
    r1[c] = cv && li1 != INT_MAX ? col[tid + NT] : 0.f;
    s2[c * LDS] = cv && li2 != INT_MAX ? col[tid + 2 * NT] : 0.f;
    s3[c * LDS] = cv && li3 != INT_MAX ? col[tid + 3 * NT] : 0.f;
  }
  __syncthreads();
  const int steps = min(nb, m);
  const int steps4 = (steps + 3) & ~3;  // register rows rotate once per step, padded steps included
#pragma unroll 1
  for (int j0 = 0; j0 < steps4; j0 += 4) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int j = j0 + u;
      if (j < steps) {
        const int buf = j & 1;
        unsigned kb = 0;
        int ib = INT_MAX;
        auto cand = [&](unsigned k, int i) {
          if (i >= j && (k > kb || (k == kb && i < ib))) {
            kb = k;
            ib = i;
          }
        };
        cand(mag_key(r0[0]), li0);
        cand(mag_key(r1[0]), li1);
        cand(mag_key(s2[j * LDS]), li2);
        cand(mag_key(s3[j * LDS]), li3);
        const unsigned kw = __reduce_max_sync(0xffffffffu, kb);
        const int iw = __reduce_min_sync(0xffffffffu, kb == kw ? ib : INT_MAX);
        if (iw != INT_MAX && ib == iw) {
          float4* dst = reinterpret_cast<float4*>(srow + (buf * NW + warp) * W);
          float v[W];
          if (li0 == iw || li1 == iw) {
            const bool z = li0 == iw;
#pragma unroll
            for (int k = 0; k < W; ++k) v[k] = k < W - j ? (z ? r0[k] : r1[k]) : 0.f;
          } else {
            const float* src = (li2 == iw ? s2 : s3) + j * LDS;
#pragma unroll
            for (int k = 0; k < W; ++k) v[k] = k < W - j ? src[k * LDS] : 0.f;
          }
#pragma unroll
          for (int k = 0; k < W / 4; ++k) dst[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
        }
        if (lane == 0) {
          skey[buf * NW + warp] = kw;
          sli[buf * NW + warp] = iw;
        }
        __syncthreads();
        const unsigned sk = lane < NW ? skey[buf * NW + lane] : 0u;
        const int si = lane < NW ? sli[buf * NW + lane] : INT_MAX;
        const unsigned kc = __reduce_max_sync(0xffffffffu, sk);
        const int ic = __reduce_min_sync(0xffffffffu, sk == kc ? si : INT_MAX);
        const unsigned wm = __ballot_sync(0xffffffffu, lane < NW && si == ic && ic != INT_MAX);
        const int wwin = wm ? __ffs(wm) - 1 : 0;
        const int piv = ic == INT_MAX ? j : ic;
        const float4* p4 = reinterpret_cast<const float4*>(srow + (buf * NW + wwin) * W);
        float pv[W];
#pragma unroll
        for (int k = 0; k < W / 4; ++k) {
          const float4 t = p4[k];
          pv[4 * k] = t.x;
          pv[4 * k + 1] = t.y;
          pv[4 * k + 2] = t.z;
          pv[4 * k + 3] = t.w;
        }
        if (tid == 0) ipiv[k0 + j] = k0 + piv;
        const bool ok = ic != INT_MAX && mag_key(pv[0]) != 0;
        if (!ok && tid == 0 && info && *info == 0) *info = k0 + j + 1;
        auto relabel = [&](int& x) {
          if (x == INT_MAX) return;
          if (x == piv)
            x = j;
          else if (x == j)
            x = piv;
        };
        relabel(li0);
        relabel(li1);
        relabel(li2);
        relabel(li3);
        if (ok) {
          const float rd = recip_newton(pv[0]);
          if (li0 > j && li0 != INT_MAX) {
            const float l = r0[0] * rd;
            r0[0] = l;
#pragma unroll
            for (int k = 1; k < W; ++k) r0[k] -= l * pv[k];
          }
          if (li1 > j && li1 != INT_MAX) {
            const float l = r1[0] * rd;
            r1[0] = l;
#pragma unroll
            for (int k = 1; k < W; ++k) r1[k] -= l * pv[k];
          }
          if (li2 > j && li2 != INT_MAX) {
            const float l = s2[j * LDS] * rd;
            s2[j * LDS] = l;
            smem_row_update<LDS>(s2, j, l, pv);
          }
          if (li3 > j && li3 != INT_MAX) {
            const float l = s3[j * LDS] * rd;
            s3[j * LDS] = l;
            smem_row_update<LDS>(s3, j, l, pv);
          }
        }
      }
      // rotate the register rows by one (padded steps rotate too)
      const float t0 = r0[0], t1 = r1[0];
#pragma unroll
      for (int k = 0; k < W - 1; ++k) {
        r0[k] = r0[k + 1];
        r1[k] = r1[k + 1];
      }
      r0[W - 1] = t0;
      r1[W - 1] = t1;
    }
  }
  __syncthreads();
  // r[k] holds column (k + steps4) mod W
#pragma unroll
  for (int k = 0; k < W; ++k) {
    const int c = (k + steps4) & (W - 1);
    if (c >= nb) continue;
    float* col = A + (size_t)(k0 + c) * lda + k0;
    if (li0 != INT_MAX) col[li0] = r0[k];
    if (li1 != INT_MAX) col[li1] = r1[k];
  }
  for (int c = 0; c < nb; ++c) {
    float* col = A + (size_t)(k0 + c) * lda + k0;
    if (li2 != INT_MAX) col[li2] = s2[c * LDS];
    if (li3 != INT_MAX) col[li3] = s3[c * LDS];
  }
  if (gath) {
    // the panel's interchanges as a gather: (destination, source) rows of every
    // row that moved -- at most 2 nb of them
    __shared__ int gcnt;
    if (tid == 0) gcnt = 0;
    __syncthreads();
    auto emit = [&](int li, int ph) {
      if (li != INT_MAX && li != ph) {
        const int t = atomicAdd(&gcnt, 1);
        if (t < 2 * kNB) {
          gath[1 + 2 * t] = k0 + li;
          gath[2 + 2 * t] = k0 + ph;
        }
      }
    };
    emit(li0, tid);
    emit(li1, tid + NT);
    emit(li2, tid + 2 * NT);
    emit(li3, tid + 3 * NT);
    __syncthreads();
    if (tid == 0) gath[0] = gcnt < 2 * kNB ? gcnt : 2 * kNB;
  }
  if (linv && nb <= m) {
    constexpr int ldx = W + 1;
#pragma unroll
    for (int k = 0; k < W; ++k) {
      const int c = (k + steps4) & (W - 1);
      if (c >= nb) continue;
      if (li0 < nb) Ls[li0 + c * ldx] = r0[k];
      if (li1 < nb) Ls[li1 + c * ldx] = r1[k];
    }
    for (int c = 0; c < nb; ++c) {
      if (li2 < nb) Ls[li2 + c * ldx] = s2[c * LDS];
      if (li3 < nb) Ls[li3 + c * ldx] = s3[c * LDS];
    }
    __syncthreads();
    constexpr int kCols = 4;
    for (int c0 = warp * kCols; c0 < nb; c0 += NW * kCols) {
      float x[kCols];
#pragma unroll
      for (int q = 0; q < kCols; ++q) x[q] = lane == c0 + q ? 1.f : 0.f;
      for (int k = c0; k < nb - 1; ++k) {
        const float lik = lane > k && lane < nb ? Ls[lane + k * ldx] : 0.f;
#pragma unroll
        for (int q = 0; q < kCols; ++q) {
          const float xk = __shfl_sync(0xffffffffu, x[q], k);
          x[q] -= lik * xk;
        }
      }
#pragma unroll
      for (int q = 0; q < kCols; ++q)
        if (c0 + q < nb && lane < nb) Xs[lane + (c0 + q) * ldx] = x[q];
    }
    __syncthreads();
    for (int idx = tid; idx < nb * nb; idx += NT) linv[idx] = Xs[(idx % nb) + (idx / nb) * ldx];
  }
}

namespace {
// Panel factorization: an FP32 panel of up to kPanelCtaMaxRows rows in one CTA
// (kind 0), else distributed shared memory of one 16-CTA (or 8-CTA) cluster
// (one panel row per thread) when the panel fits, the global-memory kernel
// otherwise.
template <typename T>
int panel_factor(cudaStream_t s, T* A, int lda, int n, int k0, int nb, int* ipiv, int* info, T* linv,
                 bool* linv_done, int kind, int* gath = nullptr, bool* gath_done = nullptr) {
  *linv_done = false;
  if (gath_done) *gath_done = false;
  const int m = n - k0;
  if constexpr (std::is_same<T, float>::value) {
    // measured per panel on GB300 (32 columns): the cluster kernel ~69 us at any
    // height; one CTA 75 us at 2000 rows, 65 at 1500, 59 at 1000, 43 at 500 (256
    // threads), 36 at 100 (128 threads)
    if (kind == 0 && m <= kPanelCtaMaxRows && m >= nb && nb <= kNB) {
      if (m > 512) {
        SLAB_TRY(ensure_smem(biglu_panel_cta_kernel<512>, panel_cta_smem_bytes<512>(), "biglu_panel_cta"));
        biglu_panel_cta_kernel<512><<<1, 512, panel_cta_smem_bytes<512>(), s>>>(A, lda, n, k0, nb, ipiv, info, linv,
                                                                                  gath);
      } else if (m > 256) {
        SLAB_TRY(ensure_smem(biglu_panel_cta_kernel<256>, panel_cta_smem_bytes<256>(), "biglu_panel_cta"));
        biglu_panel_cta_kernel<256><<<1, 256, panel_cta_smem_bytes<256>(), s>>>(A, lda, n, k0, nb, ipiv, info, linv,
                                                                                  gath);
      } else {
        SLAB_TRY(ensure_smem(biglu_panel_cta_kernel<128>, panel_cta_smem_bytes<128>(), "biglu_panel_cta"));
        biglu_panel_cta_kernel<128><<<1, 128, panel_cta_smem_bytes<128>(), s>>>(A, lda, n, k0, nb, ipiv, info, linv,
                                                                                  gath);
      }
      SLAB_CHECK_LAUNCH();
      *linv_done = linv != nullptr;
      if (gath_done) *gath_done = gath != nullptr;
      return SLAB_OK;
    }
  }
  const void* kern = reinterpret_cast<const void*>(biglu_panel_cluster_kernel<T>);
  const size_t lim = allow_dynamic_smem(kern);
  int CL = cluster_size_for(kern, panel_cluster_smem_bytes(m, nb, ceil_div(m, 16), sizeof(T)), 256);
  int R = ceil_div(m, CL);
  size_t bytes = panel_cluster_smem_bytes(m, nb, R, sizeof(T));
  if (bytes <= lim && m >= CL && m >= nb && R <= 256 && CL <= 16 && nb <= kNB) {
    void* args[] = {(void*)&A, (void*)&lda, (void*)&n, (void*)&k0, (void*)&nb, (void*)&R, (void*)&ipiv,
                    (void*)&info, (void*)&linv};
    SLAB_TRY(launch_cluster(kern, CL, 256, bytes, s, args));
    *linv_done = linv != nullptr;
    return SLAB_OK;
  }
  biglu_panel_kernel<T><<<1, 1024, 0, s>>>(A, lda, n, k0, nb, ipiv, info);
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}
}  // namespace

template <typename T>
int tri_inv_blocks(cudaStream_t s, const T* LU, int lda, int n, int bs, T* Linv, T* Uinv) {
  const int nblk = ceil_div(n, bs);
  const size_t bytes = (2 * (size_t)bs * (bs + 1) + bs) * sizeof(T);
  SLAB_TRY(ensure_smem(tri_inv_blocks_kernel<T>, bytes, "tri_inv_blocks"));
  if (Linv) {
    tri_inv_blocks_kernel<T><<<nblk, 128, bytes, s>>>(LU, lda, n, bs, 0, Linv);
    SLAB_CHECK_LAUNCH();
  }
  if (Uinv) {
    tri_inv_blocks_kernel<T><<<nblk, 128, bytes, s>>>(LU, lda, n, bs, 1, Uinv);
    SLAB_CHECK_LAUNCH();
  }
  return SLAB_OK;
}

template <typename T>
int trsm_inv(cudaStream_t s, const T* Inv, int bs, int k0, int nb, T* X, int ldx, int ncols) {
  if (ncols <= 0 || nb <= 0) return SLAB_OK;
  const size_t bytes = ((size_t)bs * bs + (size_t)bs * kTrsmCols) * sizeof(T);
  SLAB_TRY(ensure_smem(trsm_inv_kernel<T>, bytes, "trsm_inv"));
  trsm_inv_kernel<T><<<ceil_div(ncols, kTrsmCols), 256, bytes, s>>>(Inv, bs, k0, nb, X, ldx, ncols);
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}

template <typename T>
int biglu_panel_swap(cudaStream_t s, T* A, int lda, int n, int k0, int nb, int* ipiv, int* info, T* linv,
                     bool* linv_done) {
  SLAB_TRY(panel_factor<T>(s, A, lda, n, k0, nb, ipiv, info, linv, linv_done, 0));
  if (n - nb > 0) {
    biglu_swap_kernel<T><<<ceil_div(n - nb, 256), 256, 0, s>>>(A, lda, n, k0, nb, ipiv);
    SLAB_CHECK_LAUNCH();
  }
  return SLAB_OK;
}
template <typename T>
int biglu_panel_swap_range(cudaStream_t s, T* A, int lda, int n, int k0, int nb, int c_lo, int c_hi, int* ipiv,
                           int* info, T* linv, bool* linv_done) {
  SLAB_TRY(panel_factor<T>(s, A, lda, n, k0, nb, ipiv, info, linv, linv_done, 0));
  const int ncols = (c_hi - c_lo) - nb;  // the panel lies inside [c_lo, c_hi)
  if (ncols > 0) {
    swap_cols_kernel<T><<<ceil_div(ncols, 128), 128, 0, s>>>(A, lda, c_lo, c_hi, k0, nb, ipiv);
    SLAB_CHECK_LAUNCH();
  }
  return SLAB_OK;
}
template int biglu_panel_swap_range<double>(cudaStream_t, double*, int, int, int, int, int, int, int*, int*, double*,
                                            bool*);

__global__ void rowperm_build_kernel(const int* ipiv, int k0, int npiv, int n, int* out) {
  extern __shared__ int src[];  // src[i]: source row of row k0 + i
  __shared__ int cnt;
  const int m = n - k0;
  for (int i = threadIdx.x; i < m; i += blockDim.x) src[i] = k0 + i;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int j = 0; j < npiv; ++j) {
      const int a = j, b = ipiv[k0 + j] - k0;
      if (b != a && b >= 0 && b < m) {
        const int t = src[a];
        src[a] = src[b];
        src[b] = t;
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    if (src[i] != k0 + i) {
      const int t = atomicAdd(&cnt, 1);
      if (t < kRowpermMax) {
        out[1 + 2 * t] = k0 + i;
        out[2 + 2 * t] = src[i];
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) out[0] = cnt < kRowpermMax ? cnt : kRowpermMax;
}

template <typename T>
int laswp_gather(cudaStream_t s, T* A, int lda, int n, int k0, int npiv, const int* ipiv, int lo1, int hi1, int lo2,
                 int hi2, int* perm) {
  if (npiv <= 0) return SLAB_OK;
  if (2 * npiv > kRowpermMax) return set_error(SLAB_ERR_ARG, "laswp_gather: %d interchanges exceed %d", npiv, kRowpermMax / 2);
  const int ncols = max(0, hi1 - lo1) + max(0, hi2 - lo2);
  if (ncols <= 0) return SLAB_OK;
  const size_t bytes = (size_t)(n - k0) * sizeof(int);
  SLAB_TRY(ensure_smem(rowperm_build_kernel, bytes, "laswp_gather"));
  rowperm_build_kernel<<<1, 256, bytes, s>>>(ipiv, k0, npiv, n, perm);
  SLAB_CHECK_LAUNCH();
  rowperm_apply_kernel<T><<<ceil_div(ncols, kRowpermCols), 256, 0, s>>>(A, lda, lo1, hi1, lo2, hi2, perm);
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}
template int laswp_gather<double>(cudaStream_t, double*, int, int, int, int, const int*, int, int, int, int, int*);
template int laswp_gather<float>(cudaStream_t, float*, int, int, int, int, const int*, int, int, int, int, int*);

template int biglu_panel_swap<float>(cudaStream_t, float*, int, int, int, int, int*, int*, float*, bool*);
template int biglu_panel_swap<double>(cudaStream_t, double*, int, int, int, int, int*, int*, double*, bool*);

template <typename T>
int biglu(cudaStream_t s, T* A, int lda, int n, int* ipiv, int* info, T* work, int panel_kind) {
  for (int k0 = 0; k0 < n; k0 += kNB) {
    const int nb = n - k0 < kNB ? n - k0 : kNB;
    bool linv_done = false;
    SLAB_TRY(panel_factor<T>(s, A, lda, n, k0, nb, ipiv, info, work, &linv_done, panel_kind));
    if (n - nb > 0) {
      biglu_swap_kernel<T><<<ceil_div(n - nb, 256), 256, 0, s>>>(A, lda, n, k0, nb, ipiv);
      SLAB_CHECK_LAUNCH();
    }
    const int rest = n - k0 - nb;
    if (rest > 0) {
      if (work) {
        // U12 = L11^{-1} A12 through the explicit inverse of the panel's unit-lower triangle
        if (!linv_done) SLAB_TRY(tri_inv_blocks<T>(s, A + (size_t)k0 * lda + k0, lda, nb, kNB, work, nullptr));
        SLAB_TRY(trsm_inv<T>(s, work, linv_done ? nb : kNB, k0, nb, A + (size_t)(k0 + nb) * lda, lda, rest));
      } else {
        trsm_block_kernel<T><<<ceil_div(rest, 64), 256, 0, s>>>(A, lda, k0, nb, A + (size_t)(k0 + nb) * lda, lda,
                                                               rest, 0);
        SLAB_CHECK_LAUNCH();
      }
      SLAB_TRY(gemm<T>(s, rest, rest, nb, T(-1), A + (size_t)k0 * lda + k0 + nb, nullptr, 0, lda,
                       A + (size_t)(k0 + nb) * lda + k0, nullptr, 0, lda, T(1),
                       A + (size_t)(k0 + nb) * lda + k0 + nb, nullptr, 0, lda, 1));
    }
  }
  return SLAB_OK;
}

// A22 -= A21 L11^{-1} A12 for the nc columns c0.. of an outer block [ob0, obe):
// U12 = L11^{-1} A12 block by block (inverted 64 x 64 diagonal triangles of the
// unit-lower L11 in blk_linv, products below them inside the block), then one
// (n - obe) x nc x (obe - ob0) product for the rows below the block.
template <typename T>
int outer_block_update(cudaStream_t s, T* A, int lda, int n, int ob0, int obe, int c0, int nc, const T* blk_linv) {
  constexpr int kB = 64;
  if (nc <= 0) return SLAB_OK;
  T* A12 = A + (size_t)c0 * lda;
  for (int b0 = ob0; b0 < obe; b0 += kB) {
    const int bn = obe - b0 < kB ? obe - b0 : kB;
    SLAB_TRY(trsm_inv<T>(s, blk_linv + (size_t)((b0 - ob0) / kB) * kB * kB, kB, b0, bn, A12, lda, nc));
    const int below = obe - b0 - bn;
    if (below > 0)
      SLAB_TRY(gemm<T>(s, below, nc, bn, T(-1), A + (size_t)b0 * lda + b0 + bn, nullptr, 0, lda, A12 + b0, nullptr, 0,
                       lda, T(1), A12 + b0 + bn, nullptr, 0, lda, 1));
  }
  if (n - obe <= 0) return SLAB_OK;
  return gemm<T>(s, n - obe, nc, obe - ob0, T(-1), A + (size_t)ob0 * lda + obe, nullptr, 0, lda, A12 + ob0, nullptr,
                 0, lda, T(1), A12 + obe, nullptr, 0, lda, 1);
}

template <typename T>
int biglu_blocked(cudaStream_t s, T* A, int lda, int n, int* ipiv, int* info, T* panel_linv, T* blk_linv,
                  int panel_kind, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join, int* perm, int* gath) {
  constexpr int kOuter = 256, kB = 64;
  const bool look = side && fork && join && perm;
  bool side_busy = false;
  for (int ob0 = 0; ob0 < n; ob0 += kOuter) {
    const int obe = n - ob0 < kOuter ? n : ob0 + kOuter;
    for (int k0 = ob0; k0 < obe; k0 += kNB) {
      const int nb = obe - k0 < kNB ? obe - k0 : kNB;
      bool linv_done = false, gath_done = false;
      SLAB_TRY(panel_factor<T>(s, A, lda, n, k0, nb, ipiv, info, panel_linv, &linv_done, panel_kind, gath,
                               &gath_done));
      // interchanges inside the outer block now (with lookahead), the rest after it
      const int c_lo = look ? ob0 : 0, c_hi = look ? obe : n;
      const int ncols = (c_hi - c_lo) - nb;
      if (ncols > 0) {
        if (gath_done)
          swap_gather_kernel<T><<<ceil_div(ncols, 128), 128, 0, s>>>(A, lda, c_lo, c_hi, k0, nb, gath);
        else
          swap_cols_kernel<T><<<ceil_div(ncols, 128), 128, 0, s>>>(A, lda, c_lo, c_hi, k0, nb, ipiv);
        SLAB_CHECK_LAUNCH();
      }
      const int inner = obe - k0 - nb;
      if (inner > 0) {
        if (!linv_done) SLAB_TRY(tri_inv_blocks<T>(s, A + (size_t)k0 * lda + k0, lda, nb, kNB, panel_linv, nullptr));
        SLAB_TRY(trsm_inv<T>(s, panel_linv, linv_done ? nb : kNB, k0, nb, A + (size_t)(k0 + nb) * lda, lda, inner));
        SLAB_TRY(gemm<T>(s, n - k0 - nb, inner, nb, T(-1), A + (size_t)k0 * lda + k0 + nb, nullptr, 0, lda,
                         A + (size_t)(k0 + nb) * lda + k0, nullptr, 0, lda, T(1),
                         A + (size_t)(k0 + nb) * lda + k0 + nb, nullptr, 0, lda, 1));
      }
    }
    const int rest = n - obe;
    if (look) {
      // the side stream's update of the previous outer block reads the columns
      // left of ob0 and writes those right of obe: it finishes before this
      // block's interchanges reach them
      if (side_busy) SLAB_CUDA_TRY(cudaStreamWaitEvent(s, join, 0));
      side_busy = false;
      SLAB_TRY(laswp_gather<T>(s, A, lda, n, ob0, obe - ob0, ipiv, 0, ob0, obe, n, perm));
    }
    if (rest > 0) {
      SLAB_TRY(tri_inv_blocks<T>(s, A + (size_t)ob0 * lda + ob0, lda, obe - ob0, kB, blk_linv, nullptr));
      const int now = look ? (rest < kOuter ? rest : kOuter) : rest;  // the columns the next outer block needs
      SLAB_TRY(outer_block_update<T>(s, A, lda, n, ob0, obe, obe, now, blk_linv));
      if (now < rest) {
        SLAB_CUDA_TRY(cudaEventRecord(fork, s));
        SLAB_CUDA_TRY(cudaStreamWaitEvent(side, fork, 0));
        SLAB_TRY(outer_block_update<T>(side, A, lda, n, ob0, obe, obe + now, rest - now, blk_linv));
        SLAB_CUDA_TRY(cudaEventRecord(join, side));
        side_busy = true;
      }
    }
  }
  if (side_busy) SLAB_CUDA_TRY(cudaStreamWaitEvent(s, join, 0));
  return SLAB_OK;
}
template int biglu_blocked<float>(cudaStream_t, float*, int, int, int*, int*, float*, float*, int, cudaStream_t,
                                  cudaEvent_t, cudaEvent_t, int*, int*);

template <typename T>
int bigtrs_inv(cudaStream_t s, const T* LU, int lda, int n, const int* perm, const T* Linv, const T* Uinv, int bs,
               const T* B, int ldb, T* X, int ldx, int nrhs) {
  if (n <= 0 || nrhs <= 0) return SLAB_OK;
  const long long tot = (long long)n * nrhs;
  permute_rows_kernel<T><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(B, ldb, X, ldx, n, nrhs, perm);
  SLAB_CHECK_LAUNCH();
  const int nblk = ceil_div(n, bs);
  for (int b = 0; b < nblk; ++b) {
    const int k0 = b * bs, nb = n - k0 < bs ? n - k0 : bs;
    SLAB_TRY(trsm_inv<T>(s, Linv + (size_t)b * bs * bs, bs, k0, nb, X, ldx, nrhs));
    const int rest = n - k0 - nb;
    if (rest > 0)
      SLAB_TRY(gemm<T>(s, rest, nrhs, nb, T(-1), LU + (size_t)k0 * lda + k0 + nb, nullptr, 0, lda, X + k0, nullptr, 0,
                       ldx, T(1), X + k0 + nb, nullptr, 0, ldx, 1));
  }
  for (int b = nblk - 1; b >= 0; --b) {
    const int k0 = b * bs, nb = n - k0 < bs ? n - k0 : bs;
    SLAB_TRY(trsm_inv<T>(s, Uinv + (size_t)b * bs * bs, bs, k0, nb, X, ldx, nrhs));
    if (k0 > 0)
      SLAB_TRY(gemm<T>(s, k0, nrhs, nb, T(-1), LU + (size_t)k0 * lda, nullptr, 0, lda, X + k0, nullptr, 0, ldx, T(1), X,
                       nullptr, 0, ldx, 1));
  }
  return SLAB_OK;
}

template <typename T>
int bigtrs(cudaStream_t s, const T* LU, int lda, int n, const int* perm, const T* B, int ldb, T* X, int ldx,
           int nrhs, bool lower, bool upper) {
  if (n <= 0 || nrhs <= 0) return SLAB_OK;
  if (lower) {
    const long long tot = (long long)n * nrhs;
    permute_rows_kernel<T><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(B, ldb, X, ldx, n, nrhs, perm);
    SLAB_CHECK_LAUNCH();
  } else if (B != X) {
    SLAB_CUDA_TRY(cudaMemcpy2DAsync(X, (size_t)ldx * sizeof(T), B, (size_t)ldb * sizeof(T), (size_t)n * sizeof(T),
                                    nrhs, cudaMemcpyDeviceToDevice, s));
  }
  const int ctiles = ceil_div(nrhs, 64);
  if (lower) {
    for (int k0 = 0; k0 < n; k0 += kNB) {
      const int nb = n - k0 < kNB ? n - k0 : kNB;
      trsm_block_kernel<T><<<ctiles, 256, 0, s>>>(LU, lda, k0, nb, X, ldx, nrhs, 0);
      SLAB_CHECK_LAUNCH();
      const int rest = n - k0 - nb;
      if (rest > 0)
        SLAB_TRY(gemm<T>(s, rest, nrhs, nb, T(-1), LU + (size_t)k0 * lda + k0 + nb, nullptr, 0, lda, X + k0,
                         nullptr, 0, ldx, T(1), X + k0 + nb, nullptr, 0, ldx, 1));
    }
  }
  if (upper) {
    const int klast = ((n - 1) / kNB) * kNB;
    for (int k0 = klast; k0 >= 0; k0 -= kNB) {
      const int nb = n - k0 < kNB ? n - k0 : kNB;
      trsm_block_kernel<T><<<ctiles, 256, 0, s>>>(LU, lda, k0, nb, X, ldx, nrhs, 1);
      SLAB_CHECK_LAUNCH();
      if (k0 > 0)
        SLAB_TRY(gemm<T>(s, k0, nrhs, nb, T(-1), LU + (size_t)k0 * lda, nullptr, 0, lda, X + k0, nullptr, 0, ldx,
                         T(1), X, nullptr, 0, ldx, 1));
    }
  }
  return SLAB_OK;
}

#define SLAB_INSTANTIATE(T)                                                                                   \
  template int gemm<T>(cudaStream_t, int, int, int, T, const T*, const long long*, long long, int, const T*,  \
                       const long long*, long long, int, T, T*, const long long*, long long, int, int);       \
  template int getrf_batched<T>(cudaStream_t, int, int, T*, const long long*, long long, int, int*,           \
                                const long long*, long long, int*, int);                                      \
  template int getrs_batched<T>(cudaStream_t, int, int, const T*, const long long*, long long, int,           \
                                const int*, const long long*, long long, T*, const long long*, long long,     \
                                int, int, bool, bool);                                                        \
  template int biglu<T>(cudaStream_t, T*, int, int, int*, int*, T*, int);                                          \
  template int tri_inv_blocks<T>(cudaStream_t, const T*, int, int, int, T*, T*);                              \
  template int bigtrs_inv<T>(cudaStream_t, const T*, int, int, const int*, const T*, const T*, int, const T*,  \
                             int, T*, int, int);                                                              \
  template int bigtrs<T>(cudaStream_t, const T*, int, int, const int*, const T*, int, T*, int, int, bool, bool);

SLAB_INSTANTIATE(float)
SLAB_INSTANTIATE(double)

template int getrs_small<float>(cudaStream_t, int, int, const float*, const long long*, long long, int, const int*,
                                const long long*, long long, float*, const long long*, long long, int, int);
template int getrs_small<double>(cudaStream_t, int, int, const double*, const long long*, long long, int,
                                 const int*, const long long*, long long, double*, const long long*, long long, int,
                                 int);
template int trsv_coop<float>(cudaStream_t, const float*, int, int, const int*, const float*, const float*, int,
                              const float*, int, float*, int, int, bool);
template int trsv_coop<double>(cudaStream_t, const double*, int, int, const int*, const double*, const double*, int,
                               const double*, int, double*, int, int, bool);
template int trsm_inv<float>(cudaStream_t, const float*, int, int, int, float*, int, int);
template int trsm_inv<double>(cudaStream_t, const double*, int, int, int, double*, int, int);
template int trsv_cluster<float>(cudaStream_t, const float*, int, int, const int*, const float*, const float*,
                                 const float*, int, float*, int, int, bool);
template int trsv_cluster<double>(cudaStream_t, const double*, int, int, const int*, const double*, const double*,
                                  const double*, int, double*, int, int, bool);
template int getrs_small_t<float>(cudaStream_t, int, int, const float*, const long long*, long long, int, const int*,
                                  const long long*, long long, float*, const long long*, long long, int, int);
template int getrs_small_t<double>(cudaStream_t, int, int, const double*, const long long*, long long, int,
                                   const int*, const long long*, long long, double*, const long long*, long long,
                                   int, int);
template int gemm_tn<float>(cudaStream_t, int, int, int, float, const float*, const long long*, long long, int,
                            const float*, const long long*, long long, int, float, float*, const long long*,
                            long long, int, int);
template int gemm_tn<double>(cudaStream_t, int, int, int, double, const double*, const long long*, long long, int,
                             const double*, const long long*, long long, int, double, double*, const long long*,
                             long long, int, int);

// ---------------------------------------------------------------------------
// Dense FP64 LU of one n x n matrix through the C ABI (the periodic edge's Schur
// complement).  Work layout (256-byte aligned pieces): ipiv (n ints), perm (n
// ints), info (1 int), panel inverse (kNB x kNB), Linv and Uinv (ceil(n/64)
// blocks of 64 x 64 each).
namespace {
constexpr int kDenseInvBs = 64;
size_t al256d(size_t b) { return (b + 255) / 256 * 256; }
struct DenseWork {
  int *ipiv, *perm, *info;
  double *panel, *linv, *uinv;
};
DenseWork dense_work(void* w, int n) {
  unsigned char* p = static_cast<unsigned char*>(w);
  DenseWork d{};
  const size_t nblk = (size_t)(n + kDenseInvBs - 1) / kDenseInvBs;
  d.ipiv = reinterpret_cast<int*>(p);
  p += al256d((size_t)n * 4);
  d.perm = reinterpret_cast<int*>(p);
  p += al256d((size_t)n * 4);
  d.info = reinterpret_cast<int*>(p);
  p += 256;
  d.panel = reinterpret_cast<double*>(p);
  p += al256d((size_t)kNB * kNB * 8);
  d.linv = reinterpret_cast<double*>(p);
  p += al256d(nblk * kDenseInvBs * kDenseInvBs * 8);
  d.uinv = reinterpret_cast<double*>(p);
  return d;
}
}  // namespace

}  // namespace slab

extern "C" size_t slab_dense_lu_work_bytes(int n) {
  if (n <= 0) return 256;
  const size_t nblk = (size_t)(n + slab::kDenseInvBs - 1) / slab::kDenseInvBs;
  return 2 * slab::al256d((size_t)n * 4) + 256 + slab::al256d((size_t)slab::kNB * slab::kNB * 8) +
         2 * slab::al256d(nblk * slab::kDenseInvBs * slab::kDenseInvBs * 8);
}

extern "C" int slab_dense_lu(int n, double* A, int lda, void* work, size_t work_bytes, int* h_info, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (n <= 0 || !A || lda < n || !work || work_bytes < slab_dense_lu_work_bytes(n) ||
      reinterpret_cast<uintptr_t>(work) % 256 != 0)
    return slab::set_error(SLAB_ERR_ARG, "slab_dense_lu: invalid arguments");
  slab::DenseWork d = slab::dense_work(work, n);
  SLAB_CUDA_TRY(cudaMemsetAsync(d.info, 0, sizeof(int), s));
  SLAB_TRY(slab::biglu<double>(s, A, lda, n, d.ipiv, d.info, d.panel));
  SLAB_TRY(slab::build_perm(s, d.ipiv, n, d.perm));
  SLAB_TRY(slab::tri_inv_blocks<double>(s, A, lda, n, slab::kDenseInvBs, d.linv, d.uinv));
  int info = 0;
  SLAB_CUDA_TRY(cudaMemcpyAsync(&info, d.info, sizeof(int), cudaMemcpyDeviceToHost, s));
  SLAB_CUDA_TRY(cudaStreamSynchronize(s));
  if (h_info) *h_info = info;
  if (info > 0) return slab::set_error(info, "slab_dense_lu: zero pivot at column %d", info);
  return SLAB_OK;
}

extern "C" int slab_dense_lu_solve(int n, int nrhs, const double* LU, int lda, const void* work, const double* B,
                                   int ldb, double* X, int ldx, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (n <= 0 || nrhs <= 0 || !LU || !work || !B || !X || lda < n || ldb < n || ldx < n || B == X)
    return slab::set_error(SLAB_ERR_ARG, "slab_dense_lu_solve: invalid arguments");
  slab::DenseWork d = slab::dense_work(const_cast<void*>(work), n);
  return slab::bigtrs_inv<double>(s, LU, lda, n, d.perm, d.linv, d.uinv, slab::kDenseInvBs, B, ldb, X, ldx, nrhs);
}
