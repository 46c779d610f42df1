// SlabLU factor-and-solve engine for the unit-square HPS discretisation.
//
// Factorization
//   1. leaf_factor_kernel: per leaf LU of A_cc, S = -A_cc^{-1} A_cx, DtN
//      (Dirichlet faces decoupled as identity rows/columns).
//   2. Slab elimination as a multifrontal merge tree inside every slab:
//      leaves of a slab row merged left to right into strips (eliminating the
//      vertical faces), then strips merged by a balanced binary tree over the
//      rows (eliminating the horizontal faces).  A merge of children A, B
//      eliminates their shared faces E:
//          M = A[E,E] + B[E,E],  W = M^{-1} [A|B][E,O],  F_parent = base - col W
//      The slab root is the exact dense interface operator T = [[LL LR];[RL RR]]
//      of the slab (the reference samples it with HBS sketches,
//      src_solver/slablu_solver.py:1139-1308).
//   3. Interface block-tridiagonal system over the Npan-1 slab interfaces,
//      factored by the sequential block LU of
//      src_solver/block_tridiag_solver_structured.py:34-76:
//          S_0 = D_0,  X_j = S_j^{-1} sup_j,  S_{j+1} = D_{j+1} - sub_{j+1} X_j
//      in the interface precision (FP64 unless SLAB_PREC_FP32).
// Solve (one application of the factorization to a residual)
//   leaf forward (w = A_cc^{-1} r_c, face RHS -= Nx_c w), tree forward
//   (y = M^{-1} g_E, g_O -= col y), interface sweep, tree backward
//   (u_E = y - W u_O), leaf backward (u_c = w + S u_x).
// Refinement: FP64 residual of the full collocation system, corrections from
// the (possibly FP32) factorization, until ||du|| <= tol ||u||.
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <map>
#include <type_traits>
#include <memory>
#include <tuple>
#include <vector>

#include "leaf.cuh"
#include "ozaki.cuh"
#include "tcgemm.cuh"

namespace slab {

const char* last_error();
long long launch_count();
void add_launches(long long n);

// ---------------------------------------------------------------------------
// Device memory owner.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  int alloc(size_t b) {
    release();
    if (b == 0) return SLAB_OK;
    cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) {
      p = nullptr;
      return set_error(SLAB_ERR_ALLOC, "cudaMalloc(%zu) failed: %s", b, cudaGetErrorString(e));
    }
    bytes = b;
    return SLAB_OK;
  }
  int ensure(size_t b) { return b <= bytes ? SLAB_OK : alloc(b); }
  template <typename U>
  U* as() const {
    return static_cast<U*>(p);
  }
};

template <typename U>
static int upload(DevBuf& d, const std::vector<U>& h, cudaStream_t s) {
  SLAB_TRY(d.alloc(h.size() * sizeof(U)));
  if (!h.empty()) SLAB_CUDA_TRY(cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(U), cudaMemcpyHostToDevice, s));
  return SLAB_OK;
}

// ---------------------------------------------------------------------------
// Elementwise helper kernels.
template <typename T>
__global__ void gather_kernel(const T* __restrict__ vec, long long ldv, const int* __restrict__ glob, int len,
                              int count, int nrhs, T* __restrict__ out) {
  const long long tot = (long long)count * len * nrhs;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i % len);
    const long long ec = i / len;
    const int c = (int)(ec % nrhs);
    const long long e = ec / nrhs;
    out[i] = vec[glob[e * len + r] + (long long)c * ldv];
  }
}

template <typename T>
__global__ void scatter_add_kernel(T* vec, long long ldv, const int* __restrict__ glob, int len, int count, int nrhs,
                                   const T* __restrict__ in, T sign, const unsigned char* __restrict__ skip) {
  const long long tot = (long long)count * len * nrhs;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i % len);
    const long long ec = i / len;
    const int c = (int)(ec % nrhs);
    const long long e = ec / nrhs;
    const int g = glob[e * len + r];
    if (skip && skip[g]) continue;
    atomicAdd(&vec[g + (long long)c * ldv], sign * in[i]);
  }
}

template <typename T>
__global__ void scatter_set_kernel(T* vec, long long ldv, const int* __restrict__ glob, int len, int count, int nrhs,
                                   const T* __restrict__ in) {
  const long long tot = (long long)count * len * nrhs;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i % len);
    const long long ec = i / len;
    const int c = (int)(ec % nrhs);
    const long long e = ec / nrhs;
    vec[glob[e * len + r] + (long long)c * ldv] = in[i];
  }
}

template <typename Tout, typename Tin>
__global__ void convert_kernel(const Tin* __restrict__ in, Tout* __restrict__ out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (Tout)in[i];
}

template <typename Tin>
__global__ void axpy_kernel(double* __restrict__ y, const Tin* __restrict__ x, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] += (double)x[i];
}

// boundary values on Dirichlet face nodes, zero elsewhere
__global__ void init_faces_kernel(const double* __restrict__ bnd, const unsigned char* __restrict__ dir,
                                  double* __restrict__ ux, long long ntot, int nrhs) {
  const long long tot = ntot * nrhs;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const long long g = i % ntot;
    ux[i] = dir[g] ? bnd[i] : 0.0;
  }
}

template <typename T>
__global__ void sumsq_kernel(const T* __restrict__ x, long long n, double* __restrict__ acc) {
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double v = (double)x[i];
    s += v * v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  __shared__ double ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) atomicAdd(acc, s);
  }
}

// dst = src where the face's Dirichlet flag equals keep_dir, else 0 (ntot x nrhs).
__global__ void mask_faces_kernel(const double* __restrict__ src, const unsigned char* __restrict__ dir,
                                  double* __restrict__ dst, long long ntot, int nrhs, int keep_dir) {
  const long long tot = ntot * nrhs;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const long long g = i % ntot;
    dst[i] = ((int)dir[g] == keep_dir && src) ? src[i] : 0.0;
  }
}

// Leaf-major interior values -> leaf-node layout (nleaf*p*p x nrhs column-major),
// zero at the leaf boundary nodes.
__global__ void interior_to_nodes_kernel(const double* __restrict__ uc, double* __restrict__ out, int p, int nleaf,
                                         int nrhs) {
  const int q = p - 2, n = q * q, pp = p * p;
  const long long tot = (long long)nleaf * pp * nrhs;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const long long node = i % ((long long)nleaf * pp);
    const int c = (int)(i / ((long long)nleaf * pp));
    const int leaf = (int)(node / pp), k = (int)(node % pp);
    const int i1 = k / p, i2 = k % p;
    double v = 0.0;
    if (i1 >= 1 && i1 <= p - 2 && i2 >= 1 && i2 <= p - 2)
      v = uc[((size_t)leaf * nrhs + c) * n + (size_t)(i1 - 1) * q + (i2 - 1)];
    out[i] = v;
  }
}

static unsigned grid_for(long long n) {
  long long g = (n + 255) / 256;
  if (g > 4096) g = 4096;
  if (g < 1) g = 1;
  return (unsigned)g;
}

// Merge-tree assembly: parent F, M | row (Maug), col.
struct MergeGatherArgs {
  int nA, nB, nE, nO, count;
  const int* eA;
  const int* eB;
  const int* oChild;  // 0 = A, 1 = B
  const int* oPos;
  const long long* offA;
  const long long* offB;
  long long offP0, offM0, offC0;
};

// One warp per column of the parent front P (nO x nO), of Maug (nE x (nE + nO))
// or of col (nO x nE), the lanes down the rows: the column's source (child and
// position) is read once per warp, and no index is divided.
template <typename T>
__global__ void merge_gather_kernel(MergeGatherArgs a, const T* __restrict__ pool, T* __restrict__ ppool,
                                    T* __restrict__ fpool) {
  const int e = blockIdx.y;
  const T* A = pool + a.offA[e];
  const T* B = pool + a.offB[e];
  T* P = ppool + a.offP0 + (long long)e * a.nO * a.nO;
  T* M = fpool + a.offM0 + (long long)e * a.nE * (a.nE + a.nO);
  T* C = fpool + a.offC0 + (long long)e * a.nO * a.nE;
  const int nE = a.nE, nO = a.nO;
  const int ncol = 2 * nO + 2 * nE;  // P's columns, then Maug's, then col's
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  for (int vc = blockIdx.x * wpb + warp; vc < ncol; vc += gridDim.x * wpb) {
    if (vc < nO) {
      const int c = vc, cc = a.oChild[c];
      const T* src = cc == 0 ? A + (long long)a.oPos[c] * a.nA : B + (long long)a.oPos[c] * a.nB;
      T* dst = P + (long long)c * nO;
      for (int r = lane; r < nO; r += 32) dst[r] = a.oChild[r] == cc ? src[a.oPos[r]] : T(0);
    } else if (vc < 2 * nO + nE) {
      const int c = vc - nO;
      T* dst = M + (long long)c * nE;
      if (c < nE) {
        const T* sa = A + (long long)a.eA[c] * a.nA;
        const T* sb = B + (long long)a.eB[c] * a.nB;
        for (int r = lane; r < nE; r += 32) dst[r] = sa[a.eA[r]] + sb[a.eB[r]];
      } else {
        const int o = c - nE;
        const bool fromA = a.oChild[o] == 0;
        const T* src = fromA ? A + (long long)a.oPos[o] * a.nA : B + (long long)a.oPos[o] * a.nB;
        const int* ei = fromA ? a.eA : a.eB;
        for (int r = lane; r < nE; r += 32) dst[r] = src[ei[r]];
      }
    } else {
      const int c = vc - 2 * nO - nE;
      const T* sa = A + (long long)a.eA[c] * a.nA;
      const T* sb = B + (long long)a.eB[c] * a.nB;
      T* dst = C + (long long)c * nO;
      for (int r = lane; r < nO; r += 32) dst[r] = a.oChild[r] == 0 ? sa[a.oPos[r]] : sb[a.oPos[r]];
    }
  }
}

// Interface blocks from slab roots (root order [L | R | D | U], nR = 2 nI + extra).
template <typename TI, typename T>
__global__ void iface_gather_kernel(const T* __restrict__ pool, const long long* __restrict__ rootoff, int nR, int nI,
                                    int nb, TI* __restrict__ diag, TI* __restrict__ sub, TI* __restrict__ sup) {
  const long long blk = (long long)nI * nI;
  const long long tot = blk * nb * 3;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const int which = (int)(i / (blk * nb));
    const long long k = i % (blk * nb);
    const int j = (int)(k / blk);
    const int rc = (int)(k % blk);
    const int r = rc % nI, c = rc / nI;
    const T* Rj = pool + rootoff[j];
    const T* Rj1 = pool + rootoff[j + 1];
    if (which == 0) {
      diag[k] = (TI)Rj[(nI + r) + (long long)(nI + c) * nR] + (TI)Rj1[r + (long long)c * nR];
    } else if (which == 1) {
      if (j >= 1) sub[k] = (TI)Rj[(nI + r) + (long long)c * nR];  // block row j, column j-1
    } else {
      if (j <= nb - 2) sup[k] = (TI)Rj1[r + (long long)(nI + c) * nR];  // block row j, column j+1
    }
  }
}

// ---------------------------------------------------------------------------
// Status words of a refined solve run as one graph (capture_solve):
//   [0] completed refinement steps, [1] ||r||^2 of the current step, [2] ||r0||^2,
//   [3] ||du||^2, [4] ||u||^2, [5] relative correction of the last step,
//   [6] 1 once the correction reached tol, [7] final ||r||^2, [8] final ||r_int||^2.
constexpr int kGstatWords = 16;

// End of one refinement step inside the WHILE node: record the step, decide
// whether another one runs, and clear the accumulators of the next step.
__global__ void refine_step_kernel(cudaGraphConditionalHandle h, double* st, double tol, int max_iter) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int it = (int)st[0] + 1;
  st[0] = (double)it;
  if (it == 1) st[2] = st[1];
  const double rel = st[4] > 0.0 ? sqrt(st[3] / st[4]) : 0.0;
  st[5] = rel;
  const bool done = st[1] == 0.0 || rel <= tol;
  if (done) st[6] = 1.0;
  st[1] = st[3] = st[4] = 0.0;
  cudaGraphSetConditional(h, (!done && it < max_iter) ? 1u : 0u);
}

// Host-side plan.
struct HNode {
  long long off = -1;
  std::vector<int> faces;
};

struct HMerge {
  int A, B, P;  // node indices
  int level;
};

struct Batch {
  int level = 0, count = 0, nA = 0, nB = 0, nE = 0, nO = 0;
  std::vector<int> merges;
  DevBuf eA, eB, oChild, oPos, offA, offB, Eglob, Oglob;
  long long offP0 = 0, offM0 = 0, offC0 = 0, offPiv0 = 0, offY0 = 0;
  std::vector<long long> hoffA, hoffB;
};

struct EngineBase {
  virtual ~EngineBase() = default;
  virtual int factor(const LeafCoeffs& co) = 0;
  virtual int solve(int nrhs, const double* bnd, const double* fbody, double tol, int max_iter, double* ufaces,
                    double* uleaf, int* iters, double* stats) = 0;
  virtual int residual(int nrhs, const double* ufaces, const double* uint, const double* fbody, double* rint,
                       double* rfaces) = 0;
  virtual int apply_once(int nrhs, const double* rint, const double* rfaces, double* dint, double* dfaces) = 0;
  virtual int adjoint(int nrhs, const double* gleaf, const double* gfaces, double tol, int max_iter, double* lam_leaf,
                      double* lam_faces, double* gbnd, int* iters, double* stats) = 0;
  virtual int coeff_grad(int nrhs, const double* ufaces, const double* uleaf, const double* lam_leaf, double* g11,
                         double* g22, double* g12, double* g1, double* g2, double* g0) = 0;
  virtual size_t factor_bytes() const = 0;
  virtual size_t solve_bytes() const = 0;
  virtual int capture_solve(cudaGraph_t G, int nrhs, const double* bnd, const double* fbody, double* uleaf,
                            double tol, int max_iter) = 0;
  // iters/stats of the last launch; count: add its kernels to the launch count
  virtual int graph_status(int* iters, double* stats, bool count) = 0;
  virtual cudaStream_t stream() const = 0;
  // changes whenever a buffer that a captured solve reads is reallocated
  virtual long long epoch() const = 0;
  virtual double timing(int i) const = 0;
  virtual int set_option(int key, int value) = 0;
  virtual int get_option(int key) const = 0;
  long long ntot = 0, nleaf = 0;
};

template <typename T, typename TI>
struct EngineImpl : EngineBase {
  int p, q, n, nx, n0, n1, buf, npan;
  cudaStream_t s = nullptr;      // engine-owned stream (captured into graphs), high priority
  cudaStream_t us = nullptr;     // caller's stream
  cudaEvent_t join = nullptr;
  // interface LU lookahead: updates beyond the next outer block on a second,
  // low-priority stream (forked from and joined back into s)
  cudaStream_t side = nullptr;
  cudaEvent_t la_fork = nullptr, la_join = nullptr;
  DevBuf laPerm, ifBlkLinv;  // row-interchange gather scratch; inverted 64-row triangles of an FP32 outer block
  DevBuf ifGath;             // the current FP32 panel's interchanges as a gather list
  bool use_lookahead = true;
  cudaGraphExec_t gfac[3] = {nullptr, nullptr, nullptr}, gapp = nullptr, gapp_t = nullptr;
  int gapp_nrhs = 0, gapp_t_nrhs = 0;
  bool use_graphs = true;
  bool use_cluster_solve = true;
  int panel_kind = 0;  // SLAB_OPT_IFACE_PANEL
  int gemm_tiles = 0;  // SLAB_OPT_GEMM_TILES
  // FP32 interface blocks: 1 factors them with the unblocked biglu (SLAB_IFACE_UNBLOCKED=1,
  // for comparison) instead of biglu_blocked
  bool unblocked_iface = false;
  int leaf_ctas = 0;  // resident leaves per SM in the leaf kernel (0: as many as fit)
  bool leaf_split_asm = false;  // leaf operators assembled by a kernel of their own (no c12)
  DevBuf D, Dsq, Nx, NxcT, NxxT, interp, jxr, leafglob, dirmask;
  DevBuf ispan;  // per Interp_mat row: [first, last + 1) nonzero column
  DevBuf coef[6];  // c11, c22, c1, c2, c, c12
  bool has[6] = {false, false, false, false, false, false};
  // leaf factors: LU of A_cc and S in G, n x (n + ncolG) per leaf; with a mixed
  // derivative (c12) the extra columns are the 4(p-1) Jxreorder nodes
  DevBuf G, piv, leafperm, leafinfo;
  bool mixed = false;
  int ncolG = 0;
  long long leaf_stride = 0;
  DevBuf interpT;  // Interp_mat in the leaf type (mixed derivative)
  // tree
  std::vector<HNode> nodes;
  std::vector<HMerge> merges;
  std::vector<std::unique_ptr<Batch>> batches;
  DevBuf nodepool, fpool, pivpool, permpool, mergeinfo;
  long long nodepool_elems = 0, fpool_elems = 0, pivpool_elems = 0;
  std::vector<int> roots;
  DevBuf rootoff;
  int nR = 0;
  // interface
  int nI = 0, nbI = 0;
  DevBuf ifLU, ifPiv, ifPerm, ifX, ifSub, ifSup, ifInfo, ifGlob, ifLinv, ifUinv, ifWork;
  DevBuf emuWork, emuErr, emuLinv;  // tensor-core FP64 products of the interface (mixed precision)
  // inverses of the 256-row diagonal blocks of each interface LU, so that the
  // Schur right-hand sides X_j = S_j^{-1} sup_j are all tensor-core products
  DevBuf ifLoInv, ifUoInv, emuY, emuT;
  bool use_outer_inv = true;
  int nOB = 0;
  // Solve-phase copies of the interface factors in the leaf/tree type T (mixed
  // precision: FP32 copies of the FP64 factors; every correction is applied
  // through FP32 leaf and tree factors anyway, and the residual stays FP64).
  DevBuf sLU, sLinv, sUinv, sX, sSub;
  static constexpr bool kSplitSolve = !std::is_same<T, TI>::value;
  bool use_emu = false;
  // FP32 merge tree on the tensor cores: the Schur update F_parent -= col W by
  // gemm_tf32s (W = M^{-1} R stays a pivoted triangular solve)
  bool use_tc_tree = false;
  static constexpr int kTcMinE = 32;  // merges with fewer eliminated unknowns stay on the CUDA cores
  DevBuf tcWork, tcErr;
  static constexpr int kInvBs = 64;  // diagonal-block size of the interface triangular inverses
  int nInvBlk = 0;
  // solve buffers
  int cap_nrhs = 0;
  long long epoch_ = 0;
  DevBuf wc, flux, gvec, uvec, Ybuf, Zbuf, ifF, ifZ, ux_d, uc_d, rc_d, rx_d, rcT, acc;
  DevBuf gi_d, gf_d;  // adjoint right-hand side (interior leaf-major, faces)
  size_t factor_bytes_ = 0;
  size_t solve_bytes_ = 0;
  bool factored = false;
  // phase timing (CUDA events on the engine stream), milliseconds
  cudaEvent_t ev[8] = {};
  double tms[8] = {0, 0, 0, 0, 0, 0, 0, 0};

  ~EngineImpl() override {
    if (s) cudaStreamSynchronize(s);
    for (auto& g : gfac)
      if (g) cudaGraphExecDestroy(g);
    if (gapp) cudaGraphExecDestroy(gapp);
    if (gapp_t) cudaGraphExecDestroy(gapp_t);
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    if (join) cudaEventDestroy(join);
    if (la_fork) cudaEventDestroy(la_fork);
    if (la_join) cudaEventDestroy(la_join);
    if (side) {
      cudaStreamSynchronize(side);
      cudaStreamDestroy(side);
    }
    if (s) cudaStreamDestroy(s);
  }
  // order the engine stream after the caller's stream (and back)
  int enter() {
    set_gemm_tiles(gemm_tiles);
    SLAB_CUDA_TRY(cudaEventRecord(join, us));
    SLAB_CUDA_TRY(cudaStreamWaitEvent(s, join, 0));
    return SLAB_OK;
  }
  int leave() {
    set_gemm_tiles(0);
    SLAB_CUDA_TRY(cudaEventRecord(join, s));
    SLAB_CUDA_TRY(cudaStreamWaitEvent(us, join, 0));
    return SLAB_OK;
  }
  // Run `body` on the engine stream, through a CUDA graph captured on first use.
  std::map<cudaGraphExec_t, long long> graph_kernels;  // kernels captured per graph
  template <typename F>
  int run_graph(cudaGraphExec_t& exec, F body) {
    if (!use_graphs) return body();
    if (!exec) {
      cudaGraph_t g = nullptr;
      const long long before = launch_count();
      SLAB_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
      const int st = body();
      const long long captured = launch_count() - before;
      add_launches(-captured);  // counted when the graph runs, below
      const cudaError_t ce = cudaStreamEndCapture(s, &g);
      if (st != SLAB_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
      }
      if (ce != cudaSuccess) return set_error(SLAB_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
      // node priorities: the lookahead's side-stream work yields SMs to the panels
      const cudaError_t ie = cudaGraphInstantiate(&exec, g, cudaGraphInstantiateFlagUseNodePriority);
      cudaGraphDestroy(g);
      if (ie != cudaSuccess) {
        exec = nullptr;
        return set_error(SLAB_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ie));
      }
      graph_kernels[exec] = captured;
    }
    SLAB_CUDA_TRY(cudaGraphLaunch(exec, s));
    add_launches(graph_kernels[exec]);
    return SLAB_OK;
  }
  float elapsed(int a, int b) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ev[a], ev[b]) != cudaSuccess) {
      cudaGetLastError();  // timing is advisory: do not leave the error for the next check
      return -1.f;
    }
    return ms;
  }
  double timing(int i) const override { return i >= 0 && i < 8 ? tms[i] : 0.0; }

  // Tunable launch choices (see include/slablu_gb300.h); a change drops the CUDA
  // graphs that captured the old choice.
  int set_option(int key, int value) override {
    if (key == SLAB_OPT_LEAF_CTAS) {
      if (value < 0 || value > 32) return set_error(SLAB_ERR_ARG, "leaf_ctas %d out of range", value);
      if (value != leaf_ctas && gfac[0]) {
        cudaGraphExecDestroy(gfac[0]);
        gfac[0] = nullptr;
      }
      leaf_ctas = value;
      return SLAB_OK;
    }
    if (key == SLAB_OPT_IFACE_LOOKAHEAD) {
      if (value != 0 && value != 1) return set_error(SLAB_ERR_ARG, "iface_lookahead %d not 0 or 1", value);
      if ((value == 1) != use_lookahead && gfac[2]) {
        cudaGraphExecDestroy(gfac[2]);
        gfac[2] = nullptr;
      }
      use_lookahead = value == 1;
      return SLAB_OK;
    }
    if (key == SLAB_OPT_IFACE_SOLVE) {
      if (value != 0 && value != 1) return set_error(SLAB_ERR_ARG, "iface_solve %d not 0 or 1", value);
      const bool cl = value == 0;
      if (cl != use_cluster_solve) {
        for (cudaGraphExec_t* gp : {&gapp, &gapp_t})
          if (*gp) {
            cudaGraphExecDestroy(*gp);
            *gp = nullptr;
          }
      }
      use_cluster_solve = cl;
      return SLAB_OK;
    }
    if (key == SLAB_OPT_IFACE_OUTER_INV) {
      if (value != 0 && value != 1) return set_error(SLAB_ERR_ARG, "iface_outer_inv %d not 0 or 1", value);
      if ((value == 1) != use_outer_inv && gfac[2]) {
        cudaGraphExecDestroy(gfac[2]);
        gfac[2] = nullptr;
      }
      use_outer_inv = value == 1;
      return SLAB_OK;
    }
    if (key == SLAB_OPT_LEAF_ASSEMBLY) {
      if (value != 0 && value != 1) return set_error(SLAB_ERR_ARG, "leaf_assembly %d not 0 or 1", value);
      if ((value == 1) != leaf_split_asm && gfac[0]) {
        cudaGraphExecDestroy(gfac[0]);
        gfac[0] = nullptr;
      }
      leaf_split_asm = value == 1;
      return SLAB_OK;
    }
    if (key == SLAB_OPT_TREE_TC) {
      if (value != 0 && value != 1) return set_error(SLAB_ERR_ARG, "tree_tc %d not 0 or 1", value);
      if (value == 1 && !std::is_same<T, float>::value)
        return set_error(SLAB_ERR_ARG, "tree_tc: tensor-core merges need FP32 tree factors");
      if ((value == 1) != use_tc_tree) {
        if (value == 1) SLAB_TRY(alloc_tc_tree());
        if (gfac[1]) {
          cudaGraphExecDestroy(gfac[1]);
          gfac[1] = nullptr;
        }
      }
      use_tc_tree = value == 1;
      return SLAB_OK;
    }
    if (key == SLAB_OPT_GEMM_TILES) {
      if (value != 0 && value != 1) return set_error(SLAB_ERR_ARG, "gemm_tiles %d not 0 or 1", value);
      if (value != gemm_tiles) {
        for (cudaGraphExec_t* gp : {&gfac[1], &gfac[2], &gapp, &gapp_t})
          if (*gp) {
            cudaGraphExecDestroy(*gp);
            *gp = nullptr;
          }
      }
      gemm_tiles = value;
      return SLAB_OK;
    }
    if (key == SLAB_OPT_IFACE_PANEL) {
      if (value != 0 && value != 1) return set_error(SLAB_ERR_ARG, "iface_panel %d not 0 or 1", value);
      if (value != panel_kind && gfac[2]) {
        cudaGraphExecDestroy(gfac[2]);
        gfac[2] = nullptr;
      }
      panel_kind = value;
      return SLAB_OK;
    }
    return set_error(SLAB_ERR_ARG, "unknown option %d", key);
  }
  int get_option(int key) const override {
    if (key == SLAB_OPT_IFACE_PANEL) return panel_kind;
    if (key == SLAB_OPT_GEMM_TILES) return gemm_tiles;
    if (key == SLAB_OPT_TREE_TC) return use_tc_tree ? 1 : 0;
    if (key == SLAB_OPT_LEAF_ASSEMBLY) return leaf_split_asm ? 1 : 0;
    if (key == SLAB_OPT_IFACE_OUTER_INV) return use_outer_inv ? 1 : 0;
    if (key == SLAB_OPT_LEAF_CTAS) return leaf_ctas;
    if (key == SLAB_OPT_IFACE_SOLVE) return use_cluster_solve ? 0 : 1;
    if (key == SLAB_OPT_IFACE_LOOKAHEAD) return use_lookahead ? 1 : 0;
    return set_error(SLAB_ERR_ARG, "unknown option %d", key);
  }

  EngineImpl(int p_, int n0_, int n1_, int buf_, cudaStream_t s_, bool mixed_ = false)
      : p(p_), q(p_ - 2), n((p_ - 2) * (p_ - 2)), nx(4 * (p_ - 2)), n0(n0_), n1(n1_), buf(buf_), npan(n0_ / buf_),
        us(s_) {
    mixed = mixed_;
    const char* ng = getenv("SLAB_NO_GRAPHS");
    use_graphs = !(ng && ng[0] == '1');
    const char* nc = getenv("SLAB_COOP_SOLVE");  // 1: grid-wide cooperative interface solve instead of the cluster one
    use_cluster_solve = !(nc && nc[0] == '1');
    const char* lc = getenv("SLAB_LEAF_CTAS");
    if (lc) leaf_ctas = atoi(lc);
    const char* ub = getenv("SLAB_IFACE_UNBLOCKED");
    unblocked_iface = ub && ub[0] == '1';
    const char* ip = getenv("SLAB_IFACE_PANEL");  // 1: cluster panels for the FP32 interface
    if (ip) panel_kind = ip[0] == '1' ? 1 : 0;
    const char* la = getenv("SLAB_LEAF_ASSEMBLY");  // 1: assembly by a kernel of its own
    if (la) leaf_split_asm = la[0] == '1';
    const char* oi = getenv("SLAB_IFACE_OUTER_INV");  // 0: FP64-core triangular solves of 64-row blocks
    if (oi) use_outer_inv = oi[0] == '1';
    // FP64 interface products on the tensor cores in the mixed mode (FP32 leaves and
    // tree, FP64 interface); SLAB_NATIVE_FP64=1 keeps them on the FP64 cores
    const char* nf = getenv("SLAB_NATIVE_FP64");
    use_emu = std::is_same<T, float>::value && std::is_same<TI, double>::value && !(nf && nf[0] == '1');
    // 1: the FP32 merge tree's Schur updates on the tensor cores.  Off by default:
    // at N = 4.4M it shortens the tree by 3 ms but its looser FP32 accumulation
    // costs one more refinement application (6 ms); the autotuner decides.
    const char* tt = getenv("SLAB_TREE_TC");
    use_tc_tree = std::is_same<T, float>::value && tt && tt[0] == '1';
    ntot = (long long)q * ((long long)n0 * (2 * n1 + 1) + n1);
    nleaf = (long long)n0 * n1;
  }

  int faceL(int I, int J) const { return (2 * n1 + 1) * I + J; }
  int faceR(int I, int J) const { return (2 * n1 + 1) * (I + 1) + J; }
  int faceD(int I, int J) const { return (2 * n1 + 1) * I + n1 + J; }
  int faceU(int I, int J) const { return (2 * n1 + 1) * I + n1 + J + 1; }

  int add_node(std::vector<int> faces) {
    HNode h;
    h.faces = std::move(faces);
    nodes.push_back(std::move(h));
    return (int)nodes.size() - 1;
  }

  std::vector<int> strip_faces(int I0, int I1, int J) const {  // columns I0..I1 inclusive
    std::vector<int> f{faceL(I0, J), faceR(I1, J)};
    for (int I = I0; I <= I1; ++I) f.push_back(faceD(I, J));
    for (int I = I0; I <= I1; ++I) f.push_back(faceU(I, J));
    return f;
  }

  std::vector<int> range_faces(int s_, int lo, int hi) const {
    const int c0 = s_ * buf, c1 = c0 + buf - 1;
    std::vector<int> f;
    for (int J = lo; J < hi; ++J) f.push_back(faceL(c0, J));
    for (int J = lo; J < hi; ++J) f.push_back(faceR(c1, J));
    for (int I = c0; I <= c1; ++I) f.push_back(faceD(I, lo));
    for (int I = c0; I <= c1; ++I) f.push_back(faceU(I, hi - 1));
    return f;
  }

  int build_range(int s_, int lo, int hi, std::vector<int>& strip_of_row, std::vector<int>& height) {
    if (hi - lo == 1) return strip_of_row[lo];
    const int mid = lo + (hi - lo) / 2;
    const int a = build_range(s_, lo, mid, strip_of_row, height);
    const int b = build_range(s_, mid, hi, strip_of_row, height);
    const int P = add_node(range_faces(s_, lo, hi));
    height.resize(nodes.size(), 0);
    height[P] = 1 + std::max(height[a], height[b]);
    merges.push_back({a, b, P, (buf - 1) + height[P]});
    return P;
  }

  int build_plan() {
    // leaves
    for (int I = 0; I < n0; ++I)
      for (int J = 0; J < n1; ++J) {
        const int id = add_node({faceL(I, J), faceR(I, J), faceD(I, J), faceU(I, J)});
        nodes[id].off = (long long)id * nx * nx;
      }
    std::vector<int> height(nodes.size(), 0);
    for (int sl = 0; sl < npan; ++sl) {
      std::vector<int> strip_of_row(n1);
      for (int J = 0; J < n1; ++J) {
        const int c0 = sl * buf;
        int cur = c0 * n1 + J;
        for (int k = 1; k < buf; ++k) {
          const int leaf = (c0 + k) * n1 + J;
          const int P = add_node(strip_faces(c0, c0 + k, J));
          merges.push_back({cur, leaf, P, k});
          cur = P;
        }
        strip_of_row[J] = cur;
      }
      height.resize(nodes.size(), 0);
      roots.push_back(build_range(sl, 0, n1, strip_of_row, height));
    }
    // group merges into batches of identical shape and maps
    std::vector<int> order(merges.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return merges[x].level < merges[y].level; });
    std::map<std::tuple<int, int, int, int>, std::vector<int>> groups;  // (level, nA, nB, nO)
    std::vector<std::tuple<int, int, int, int>> keys;
    for (int mi : order) {
      const HMerge& m = merges[mi];
      auto key = std::make_tuple(m.level, (int)nodes[m.A].faces.size(), (int)nodes[m.B].faces.size(),
                                 (int)nodes[m.P].faces.size());
      if (!groups.count(key)) keys.push_back(key);
      groups[key].push_back(mi);
    }
    std::stable_sort(keys.begin(), keys.end(), [](const auto& x, const auto& y) { return std::get<0>(x) < std::get<0>(y); });
    long long node_cursor = nleaf * nx * nx;
    long long fcur = 0, pcur = 0;
    for (auto& key : keys) {
      auto& list = groups[key];
      // maps of the first entry; every entry must agree
      std::vector<int> eA, eB, oC, oP;
      bool first = true;
      auto b = std::make_unique<Batch>();
      b->level = std::get<0>(key);
      std::vector<int> Eg, Og;
      for (int mi : list) {
        const HMerge& m = merges[mi];
        const auto& fa = nodes[m.A].faces;
        const auto& fb = nodes[m.B].faces;
        const auto& fp = nodes[m.P].faces;
        std::vector<int> E, ea, eb;
        for (size_t i = 0; i < fa.size(); ++i) {
          auto it = std::find(fb.begin(), fb.end(), fa[i]);
          if (it != fb.end()) {
            E.push_back(fa[i]);
            ea.push_back((int)i);
            eb.push_back((int)(it - fb.begin()));
          }
        }
        std::vector<int> oc, op;
        for (int f : fp) {
          auto ia = std::find(fa.begin(), fa.end(), f);
          auto ib = std::find(fb.begin(), fb.end(), f);
          if (ia != fa.end() && ib == fb.end()) {
            oc.push_back(0);
            op.push_back((int)(ia - fa.begin()));
          } else if (ib != fb.end() && ia == fa.end()) {
            oc.push_back(1);
            op.push_back((int)(ib - fb.begin()));
          } else {
            return set_error(SLAB_ERR_STATE, "plan: parent face %d not owned by exactly one child", f);
          }
        }
        if (first) {
          eA = ea; eB = eb; oC = oc; oP = op;
          first = false;
        } else if (ea != eA || eb != eB || oc != oC || op != oP) {
          return set_error(SLAB_ERR_STATE, "plan: merges of one batch differ in structure");
        }
        for (int f : E)
          for (int k = 0; k < q; ++k) Eg.push_back(f * q + k);
        for (int f : fp)
          for (int k = 0; k < q; ++k) Og.push_back(f * q + k);
        b->hoffA.push_back(nodes[m.A].off);
        b->hoffB.push_back(nodes[m.B].off);
        if (nodes[m.A].off < 0 || nodes[m.B].off < 0) return set_error(SLAB_ERR_STATE, "plan: child not placed");
      }
      b->merges = list;
      b->count = (int)list.size();
      b->nA = (int)nodes[merges[list[0]].A].faces.size() * q;
      b->nB = (int)nodes[merges[list[0]].B].faces.size() * q;
      b->nE = (int)eA.size() * q;
      b->nO = (int)oC.size() * q;
      if (b->nE == 0) return set_error(SLAB_ERR_STATE, "plan: merge without shared faces");
      // node-position maps
      std::vector<int> meA, meB, moC, moP;
      for (size_t i = 0; i < eA.size(); ++i)
        for (int k = 0; k < q; ++k) {
          meA.push_back(eA[i] * q + k);
          meB.push_back(eB[i] * q + k);
        }
      for (size_t i = 0; i < oC.size(); ++i)
        for (int k = 0; k < q; ++k) {
          moC.push_back(oC[i]);
          moP.push_back(oP[i] * q + k);
        }
      b->offP0 = node_cursor;
      for (int e = 0; e < b->count; ++e) nodes[merges[list[e]].P].off = node_cursor + (long long)e * b->nO * b->nO;
      node_cursor += (long long)b->count * b->nO * b->nO;
      b->offM0 = fcur;
      fcur += (long long)b->count * b->nE * (b->nE + b->nO);
      b->offC0 = fcur;
      fcur += (long long)b->count * b->nO * b->nE;
      b->offPiv0 = pcur;
      pcur += (long long)b->count * b->nE;
      SLAB_TRY(upload(b->eA, meA, s));
      SLAB_TRY(upload(b->eB, meB, s));
      SLAB_TRY(upload(b->oChild, moC, s));
      SLAB_TRY(upload(b->oPos, moP, s));
      SLAB_TRY(upload(b->offA, b->hoffA, s));
      SLAB_TRY(upload(b->offB, b->hoffB, s));
      SLAB_TRY(upload(b->Eglob, Eg, s));
      SLAB_TRY(upload(b->Oglob, Og, s));
      batches.push_back(std::move(b));
    }
    nodepool_elems = node_cursor;
    fpool_elems = fcur;
    pivpool_elems = pcur;
    // roots and interface geometry
    std::vector<long long> ro;
    for (int r : roots) ro.push_back(nodes[r].off);
    nR = (int)nodes[roots[0]].faces.size() * q;
    nI = n1 * q;
    nbI = npan - 1;
    SLAB_TRY(upload(rootoff, ro, s));
    std::vector<int> ig;
    for (int j = 0; j < nbI; ++j)
      for (int J = 0; J < n1; ++J)
        for (int k = 0; k < q; ++k) ig.push_back(faceR((j + 1) * buf - 1, J) * q + k);
    SLAB_TRY(upload(ifGlob, ig, s));
    // leaf face maps and Dirichlet mask
    std::vector<int> lg((size_t)nleaf * nx);
    for (int I = 0; I < n0; ++I)
      for (int J = 0; J < n1; ++J) {
        const int l = I * n1 + J;
        const int f[4] = {faceL(I, J), faceR(I, J), faceD(I, J), faceU(I, J)};
        for (int t = 0; t < 4; ++t)
          for (int k = 0; k < q; ++k) lg[(size_t)l * nx + t * q + k] = f[t] * q + k;
      }
    SLAB_TRY(upload(leafglob, lg, s));
    std::vector<unsigned char> dm((size_t)ntot, 0);
    auto mark = [&](int f) {
      for (int k = 0; k < q; ++k) dm[(size_t)f * q + k] = 1;
    };
    for (int J = 0; J < n1; ++J) {
      mark(faceL(0, J));
      mark(faceR(n0 - 1, J));
    }
    for (int I = 0; I < n0; ++I) {
      mark(faceD(I, 0));
      mark(faceU(I, n1 - 1));
    }
    SLAB_TRY(upload(dirmask, dm, s));
    return SLAB_OK;
  }

  int init(const double* hD, const double* hDsq, const double* hNx, const double* hinterp, const int* hjxr) {
    int prio_lo = 0, prio_hi = 0;
    SLAB_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
    SLAB_CUDA_TRY(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, prio_hi));
    SLAB_CUDA_TRY(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, prio_lo));
    SLAB_CUDA_TRY(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
    SLAB_CUDA_TRY(cudaEventCreateWithFlags(&la_fork, cudaEventDisableTiming));
    SLAB_CUDA_TRY(cudaEventCreateWithFlags(&la_join, cudaEventDisableTiming));
    SLAB_TRY(upload(D, std::vector<double>(hD, hD + p * p), s));
    SLAB_TRY(upload(Dsq, std::vector<double>(hDsq, hDsq + p * p), s));
    SLAB_TRY(upload(Nx, std::vector<double>(hNx, hNx + (size_t)nx * p * p), s));
    SLAB_TRY(upload(interp, std::vector<double>(hinterp, hinterp + (size_t)4 * (p - 1) * nx), s));
    {
      // nonzero span of each Interp_mat row (one face's nodes for the reference's
      // discretisation); the assembly sums only over it
      std::vector<int> sp(2 * (size_t)4 * (p - 1));
      for (int t = 0; t < 4 * (p - 1); ++t) {
        int lo = nx, hi = 0;
        for (int c = 0; c < nx; ++c)
          if (hinterp[(size_t)t * nx + c] != 0.0) {
            lo = std::min(lo, c);
            hi = c + 1;
          }
        sp[2 * t] = lo < hi ? lo : 0;
        sp[2 * t + 1] = lo < hi ? hi : 0;
      }
      SLAB_TRY(upload(ispan, sp, s));
    }
    SLAB_TRY(upload(jxr, std::vector<int>(hjxr, hjxr + 4 * (p - 1)), s));
    SLAB_TRY(NxcT.alloc((size_t)nx * n * sizeof(T)));
    SLAB_TRY(NxxT.alloc((size_t)nx * nx * sizeof(T)));
    split_nx_kernel<T><<<64, 256, 0, s>>>(Nx.as<double>(), p, q, NxcT.as<T>(), NxxT.as<T>());
    SLAB_CHECK_LAUNCH();
    SLAB_TRY(build_plan());
    // factor storage
    ncolG = mixed ? 4 * (p - 1) : nx;
    leaf_stride = (long long)n * (n + ncolG);
    SLAB_TRY(G.alloc((size_t)nleaf * leaf_stride * sizeof(T)));
    if (mixed) {
      const long long ni = (long long)4 * (p - 1) * nx;
      SLAB_TRY(interpT.alloc((size_t)ni * sizeof(T)));
      convert_kernel<T, double><<<grid_for(ni), 256, 0, s>>>(interp.as<double>(), interpT.as<T>(), ni);
      SLAB_CHECK_LAUNCH();
    }
    SLAB_TRY(piv.alloc((size_t)nleaf * n * sizeof(int)));
    SLAB_TRY(leafperm.alloc((size_t)nleaf * n * sizeof(int)));
    SLAB_TRY(leafinfo.alloc((size_t)nleaf * sizeof(int)));
    SLAB_TRY(nodepool.alloc((size_t)nodepool_elems * sizeof(T)));
    SLAB_TRY(fpool.alloc((size_t)std::max<long long>(fpool_elems, 1) * sizeof(T)));
    SLAB_TRY(pivpool.alloc((size_t)std::max<long long>(pivpool_elems, 1) * sizeof(int)));
    SLAB_TRY(permpool.alloc((size_t)std::max<long long>(pivpool_elems, 1) * sizeof(int)));
    int ninfo = 0;
    for (auto& b : batches) ninfo += b->count;
    SLAB_TRY(mergeinfo.alloc((size_t)std::max(ninfo, 1) * sizeof(int)));
    if (nbI > 0) {
      const size_t blk = (size_t)nI * nI;
      SLAB_TRY(ifLU.alloc(blk * nbI * sizeof(TI)));
      SLAB_TRY(ifPiv.alloc((size_t)nI * nbI * sizeof(int)));
      SLAB_TRY(ifPerm.alloc((size_t)nI * nbI * sizeof(int)));
      SLAB_TRY(ifSub.alloc(blk * nbI * sizeof(TI)));
      SLAB_TRY(ifSup.alloc(blk * nbI * sizeof(TI)));
      SLAB_TRY(ifX.alloc(blk * nbI * sizeof(TI)));
      SLAB_TRY(ifInfo.alloc(sizeof(int)));
      nInvBlk = ceil_div(nI, kInvBs);
      SLAB_TRY(ifLinv.alloc((size_t)nbI * nInvBlk * kInvBs * kInvBs * sizeof(TI)));
      SLAB_TRY(ifUinv.alloc((size_t)nbI * nInvBlk * kInvBs * kInvBs * sizeof(TI)));
      SLAB_TRY(ifWork.alloc((size_t)kNB * kNB * sizeof(TI)));
      if (kSplitSolve) {
        SLAB_TRY(sLU.alloc(blk * nbI * sizeof(T)));
        SLAB_TRY(sX.alloc(blk * nbI * sizeof(T)));
        SLAB_TRY(sSub.alloc(blk * nbI * sizeof(T)));
        SLAB_TRY(sLinv.alloc((size_t)nbI * nInvBlk * kInvBs * kInvBs * sizeof(T)));
        SLAB_TRY(sUinv.alloc((size_t)nbI * nInvBlk * kInvBs * kInvBs * sizeof(T)));
      }
      if (use_emu) {
        SLAB_TRY(emuWork.alloc(dgemm_emu_work_bytes(nI, nI, nI)));
        SLAB_TRY(emuErr.alloc(sizeof(int)));
        SLAB_TRY(emuLinv.alloc((size_t)kEmuOuter * 64 * sizeof(double)));
        nOB = ceil_div(nI, kEmuOuter);
        if (nbI > 1) {
          SLAB_TRY(ifLoInv.alloc((size_t)(nbI - 1) * nOB * kEmuOuter * kEmuOuter * sizeof(double)));
          SLAB_TRY(ifUoInv.alloc((size_t)(nbI - 1) * nOB * kEmuOuter * kEmuOuter * sizeof(double)));
          SLAB_TRY(emuY.alloc((size_t)kEmuOuter * nI * sizeof(double)));
          SLAB_TRY(emuT.alloc(outer_tri_tmp_elems(nI) * sizeof(double)));
        }
        SLAB_CUDA_TRY(cudaMemsetAsync(emuErr.p, 0, sizeof(int), s));
      }
      SLAB_TRY(laPerm.alloc((size_t)(1 + 2 * kRowpermMax) * sizeof(int)));
      if (std::is_same<TI, float>::value) {
        SLAB_TRY(ifBlkLinv.alloc((size_t)kEmuOuter * 64 * sizeof(TI)));
        SLAB_TRY(ifGath.alloc((size_t)(1 + 4 * kNB) * sizeof(int)));
      }
    }
    if (use_tc_tree) SLAB_TRY(alloc_tc_tree());
    SLAB_TRY(acc.alloc(4 * sizeof(double)));
    for (auto& e : ev) SLAB_CUDA_TRY(cudaEventCreate(&e));
    SLAB_CUDA_TRY(cudaStreamSynchronize(s));
    factor_bytes_ = G.bytes + piv.bytes + leafperm.bytes + nodepool.bytes + fpool.bytes + pivpool.bytes +
                    permpool.bytes + ifLU.bytes + ifPiv.bytes + ifPerm.bytes + ifSub.bytes + ifSup.bytes + ifX.bytes +
                    ifLinv.bytes + ifUinv.bytes + sLU.bytes + sX.bytes + sSub.bytes + sLinv.bytes + sUinv.bytes;
    // factors one solve application streams: the leaf LU and S, the merge factors
    // ([M | W] and col), the interface factors it applies (LU, X, sub; the FP32
    // copies in the mixed mode) and the pivot vectors
    solve_bytes_ = G.bytes + leafperm.bytes + fpool.bytes + pivpool.bytes +
                   (kSplitSolve ? sLU.bytes + sX.bytes + sSub.bytes : ifLU.bytes + ifX.bytes + ifSub.bytes) +
                   ifPerm.bytes;
    return SLAB_OK;
  }

  size_t factor_bytes() const override { return factor_bytes_; }
  size_t solve_bytes() const override { return solve_bytes_; }

  int factor(const LeafCoeffs& co_in) override {
    SLAB_TRY(enter());
    const int st = factor_impl(co_in);
    const int st2 = leave();
    return st != SLAB_OK ? st : st2;
  }

  int factor_impl(const LeafCoeffs& co_in) {
    const size_t cbytes = (size_t)nleaf * p * p * sizeof(double);
    if ((co_in.c12 != nullptr) != mixed)
      return set_error(SLAB_ERR_ARG, mixed ? "slab_engine_factor: this engine needs the mixed-derivative coefficient c12"
                                           : "slab_engine_factor: c12 needs an engine from slab_engine_create_mixed");
    const double* src[6] = {co_in.c11, co_in.c22, co_in.c1, co_in.c2, co_in.c, co_in.c12};
    for (int i = 0; i < 6; ++i) {
      if (has[i] != (src[i] != nullptr)) ++epoch_;
      has[i] = src[i] != nullptr;
      if (has[i]) {
        if (coef[i].bytes < cbytes) ++epoch_;
        SLAB_TRY(coef[i].ensure(cbytes));
        SLAB_CUDA_TRY(cudaMemcpyAsync(coef[i].p, src[i], cbytes, cudaMemcpyDeviceToDevice, s));
      }
    }
    const bool layout_changed = !factored || has_prev[0] != has[0] || has_prev[1] != has[1] ||
                                has_prev[2] != has[2] || has_prev[3] != has[3] || has_prev[4] != has[4] ||
                                has_prev[5] != has[5];
    if (layout_changed)
      for (auto& g : gfac)
        if (g) {
          cudaGraphExecDestroy(g);
          g = nullptr;
        }
    for (int i = 0; i < 6; ++i) has_prev[i] = has[i];
    SLAB_CUDA_TRY(cudaEventRecord(ev[0], s));
    SLAB_TRY(run_graph(gfac[0], [&]() { return factor_leaf(); }));
    SLAB_CUDA_TRY(cudaEventRecord(ev[1], s));
    SLAB_TRY(run_graph(gfac[1], [&]() { return factor_tree(); }));
    SLAB_CUDA_TRY(cudaEventRecord(ev[2], s));
    if (nbI > 0) SLAB_TRY(run_graph(gfac[2], [&]() { return factor_interface(); }));
    SLAB_CUDA_TRY(cudaEventRecord(ev[3], s));
    return factor_check();
  }

  bool has_prev[6] = {false, false, false, false, false, false};

  int factor_leaf() {
    LeafCoeffs co = coeffs();
    SLAB_CUDA_TRY(cudaMemsetAsync(leafinfo.p, 0, leafinfo.bytes, s));
    SLAB_CUDA_TRY(cudaMemsetAsync(mergeinfo.p, 0, mergeinfo.bytes, s));
    LeafFactorArgs<T> a{};
    a.p = p; a.q = q; a.n = n; a.nx = nx;
    a.co = co; a.D = D.as<double>(); a.Dsq = Dsq.as<double>();
    a.Nxc = NxcT.as<T>(); a.Nxx = NxxT.as<T>();
    a.G = G.as<T>(); a.strideG = leaf_stride; a.piv = piv.as<int>();
    a.dtn = nodepool.as<T>(); a.info = leafinfo.as<int>();
    a.decouple = 1; a.n0 = n0; a.n1 = n1; a.leaf_begin = 0;
    a.preassembled = (!mixed && leaf_split_asm) ? 1 : 0;
    if (mixed) {
      a.nxa = ncolG;
      a.interp = interpT.as<T>();
      a.jxr = jxr.as<int>();
    }
    SLAB_TRY(leaf_factor<T>(s, a, (int)nleaf, leaf_ctas));
    return build_perm_batched(s, piv.as<int>(), n, n, (int)nleaf, leafperm.as<int>(), n);
  }

  // Work of the tensor-core merges: the operand slices of the largest Schur
  // product of any batch.
  int alloc_tc_tree() {
    size_t wb = 256;
    for (auto& bp : batches) {
      const Batch& b = *bp;
      if (b.nE < kTcMinE || b.nO <= 0) continue;
      wb = std::max(wb, gemm_tf32s_work_bytes(b.nO, b.nO, b.nE, b.count));
    }
    SLAB_TRY(tcWork.ensure(wb));
    SLAB_TRY(tcErr.ensure(sizeof(int)));
    SLAB_CUDA_TRY(cudaMemsetAsync(tcErr.p, 0, sizeof(int), s));
    return SLAB_OK;
  }

  int factor_tree() {
    // merge tree, level by level
    int info_ofs = 0;
    if (use_tc_tree) SLAB_CUDA_TRY(cudaMemsetAsync(tcErr.p, 0, sizeof(int), s));
    for (auto& bp : batches) {
      Batch& b = *bp;
      MergeGatherArgs g{b.nA, b.nB, b.nE, b.nO, b.count, b.eA.as<int>(), b.eB.as<int>(), b.oChild.as<int>(),
                        b.oPos.as<int>(), b.offA.as<long long>(), b.offB.as<long long>(), b.offP0, b.offM0, b.offC0};
      const long long per = (long long)b.nO * b.nO + (long long)b.nE * (b.nE + b.nO) + (long long)b.nO * b.nE;
      if (per + 1024LL * 256 >= (1LL << 31))
        return set_error(SLAB_ERR_ARG, "merge of %d + %d unknowns too large", b.nE, b.nO);
      const int ncol = 2 * b.nO + 2 * b.nE;  // one warp per column, eight per CTA
      dim3 grid((unsigned)std::max(1, std::min((ncol + 7) / 8, 1024)), b.count);
      merge_gather_kernel<T><<<grid, 256, 0, s>>>(g, nodepool.as<T>(), nodepool.as<T>(), fpool.as<T>());
      SLAB_CHECK_LAUNCH();
      T* Maug = fpool.as<T>() + b.offM0;
      const long long strideM = (long long)b.nE * (b.nE + b.nO);
      int* pv = pivpool.as<int>() + b.offPiv0;
      SLAB_TRY(getrf_batched<T>(s, b.nE, b.nE, Maug, nullptr, strideM, b.nE, pv, nullptr, b.nE,
                                mergeinfo.as<int>() + info_ofs, b.count));
      SLAB_TRY(build_perm_batched(s, pv, b.nE, b.nE, b.count, permpool.as<int>() + b.offPiv0, b.nE));
      T* R = Maug + (long long)b.nE * b.nE;
      // W = M^{-1} [A|B][E,O]: the tiled many-column substitution where M fits its shared memory
      if (getrs_many_fits<T>(b.nE))
        SLAB_TRY(getrs_many<T>(s, b.nE, b.nO, Maug, strideM, b.nE, permpool.as<int>() + b.offPiv0, b.nE, R, strideM,
                               b.nE, b.count));
      else
        SLAB_TRY(getrs_batched<T>(s, b.nE, b.nO, Maug, nullptr, strideM, b.nE, pv, nullptr, b.nE, R, nullptr, strideM,
                                  b.nE, b.count));
      bool done = false;
      if constexpr (std::is_same<T, float>::value) {
        if (use_tc_tree && b.nE >= kTcMinE && b.nO > 0) {
          // F_parent -= col W on the tensor cores (TF32-split products, FP32 error bound)
          SLAB_TRY(gemm_tf32s(s, b.nO, b.nO, b.nE, -1.f, fpool.as<T>() + b.offC0, b.nO, (long long)b.nO * b.nE, R,
                              b.nE, strideM, 1.f, nodepool.as<T>() + b.offP0, b.nO, (long long)b.nO * b.nO, b.count,
                              tcWork.p, tcWork.bytes, tcErr.as<int>()));
          done = true;
        }
      }
      if (!done)
        SLAB_TRY(gemm<T>(s, b.nO, b.nO, b.nE, T(-1), fpool.as<T>() + b.offC0, nullptr, (long long)b.nO * b.nE, b.nO,
                         R, nullptr, strideM, b.nE, T(1), nodepool.as<T>() + b.offP0, nullptr,
                         (long long)b.nO * b.nO, b.nO, b.count));
      info_ofs += b.count;
    }
    return SLAB_OK;
  }

  double* loinv(int j) { return ifLoInv.as<double>() + (size_t)j * nOB * kEmuOuter * kEmuOuter; }
  double* uoinv(int j) { return ifUoInv.as<double>() + (size_t)j * nOB * kEmuOuter * kEmuOuter; }
  TI* linv(int j) { return ifLinv.as<TI>() + (size_t)j * nInvBlk * kInvBs * kInvBs; }
  TI* uinv(int j) { return ifUinv.as<TI>() + (size_t)j * nInvBlk * kInvBs * kInvBs; }
  // solve-phase views (type T)
  size_t inv_elems() const { return (size_t)nInvBlk * kInvBs * kInvBs; }
  T* sv_of(DevBuf& split, DevBuf& full, size_t off) {
    if constexpr (kSplitSolve) return split.as<T>() + off;
    else return full.as<T>() + off;
  }
  T* luS(int j) { return sv_of(sLU, ifLU, (size_t)nI * nI * j); }
  T* xS(int j) { return sv_of(sX, ifX, (size_t)nI * nI * j); }
  T* subS(int j) { return sv_of(sSub, ifSub, (size_t)nI * nI * j); }
  T* linvS(int j) { return sv_of(sLinv, ifLinv, inv_elems() * j); }
  T* uinvS(int j) { return sv_of(sUinv, ifUinv, inv_elems() * j); }

  // FP32 copies of the FP64 interface factors for the solve phase (mixed precision).
  int split_solve_copies() {
    if constexpr (kSplitSolve) {
      const long long blk = (long long)nI * nI;
      convert_kernel<T, TI><<<grid_for(blk * nbI), 256, 0, s>>>(ifLU.as<TI>(), sLU.as<T>(), blk * nbI);
      SLAB_CHECK_LAUNCH();
      const long long ni = (long long)inv_elems() * nbI;
      convert_kernel<T, TI><<<grid_for(ni), 256, 0, s>>>(ifLinv.as<TI>(), sLinv.as<T>(), ni);
      SLAB_CHECK_LAUNCH();
      convert_kernel<T, TI><<<grid_for(ni), 256, 0, s>>>(ifUinv.as<TI>(), sUinv.as<T>(), ni);
      SLAB_CHECK_LAUNCH();
      if (nbI > 1) {
        convert_kernel<T, TI><<<grid_for(blk * (nbI - 1)), 256, 0, s>>>(ifX.as<TI>(), sX.as<T>(), blk * (nbI - 1));
        SLAB_CHECK_LAUNCH();
        convert_kernel<T, TI><<<grid_for(blk * (nbI - 1)), 256, 0, s>>>(ifSub.as<TI>() + blk, sSub.as<T>() + blk,
                                                                       blk * (nbI - 1));
        SLAB_CHECK_LAUNCH();
      }
    }
    return SLAB_OK;
  }

  // X_{j-1} = S_{j-1}^{-1} sup_{j-1}, then S_j -= sub_j X_{j-1}: on the tensor
  // cores through exact slicing when use_emu (the FP64 mixed path), else FP64 cores.
  int iface_schur(int j) {
    const long long blk = (long long)nI * nI;
    TI* Sj = ifLU.as<TI>() + blk * j;
    TI* Xprev = ifX.as<TI>() + blk * (j - 1);
    const TI* LUp = ifLU.as<TI>() + blk * (j - 1);
    const int* pp = ifPerm.as<int>() + (long long)nI * (j - 1);
    if constexpr (std::is_same<TI, double>::value) {
      if (use_emu) {
        EmuWork w{emuWork.p, emuWork.bytes, emuErr.as<int>()};
        if (use_outer_inv)
          SLAB_TRY(bigtrs_outer_emu(s, LUp, nI, nI, pp, loinv(j - 1), uoinv(j - 1), ifSup.as<TI>() + blk * (j - 1), nI,
                                    Xprev, nI, nI, emuY.as<double>(), w));
        else
          SLAB_TRY(bigtrs_inv_emu(s, LUp, nI, nI, pp, linv(j - 1), uinv(j - 1), kInvBs, ifSup.as<TI>() + blk * (j - 1),
                                  nI, Xprev, nI, nI, w));
        return dgemm_emu(s, nI, nI, nI, -1.0, ifSub.as<TI>() + blk * j, nI, Xprev, nI, 1.0, Sj, nI, w.buf, w.bytes,
                         w.err);
      }
    }
    SLAB_TRY(bigtrs_inv<TI>(s, LUp, nI, nI, pp, linv(j - 1), uinv(j - 1), kInvBs, ifSup.as<TI>() + blk * (j - 1), nI,
                            Xprev, nI, nI));
    return gemm<TI>(s, nI, nI, nI, TI(-1), ifSub.as<TI>() + blk * j, nullptr, 0, nI, Xprev, nullptr, 0, nI, TI(1), Sj,
                    nullptr, 0, nI, 1);
  }

  int factor_interface() {
    if (nbI > 0) {
      const long long blk = (long long)nI * nI;
      SLAB_CUDA_TRY(cudaMemsetAsync(ifInfo.p, 0, sizeof(int), s));
      if (use_emu) SLAB_CUDA_TRY(cudaMemsetAsync(emuErr.p, 0, sizeof(int), s));
      iface_gather_kernel<TI, T><<<grid_for(blk * nbI * 3), 256, 0, s>>>(
          nodepool.as<T>(), rootoff.as<long long>(), nR, nI, nbI, ifLU.as<TI>(), ifSub.as<TI>(), ifSup.as<TI>());
      SLAB_CHECK_LAUNCH();
      for (int j = 0; j < nbI; ++j) {
        TI* Sj = ifLU.as<TI>() + blk * j;
        if (j > 0) SLAB_TRY(iface_schur(j));
        bool done = false;
        if constexpr (std::is_same<TI, double>::value) {
          if (use_emu) {
            EmuWork w{emuWork.p, emuWork.bytes, emuErr.as<int>()};
            Lookahead la{use_lookahead ? side : nullptr, la_fork, la_join, laPerm.as<int>()};
            SLAB_TRY(biglu_emu(s, Sj, nI, nI, ifPiv.as<int>() + (long long)nI * j, ifInfo.as<int>(), ifWork.as<TI>(),
                               emuLinv.as<double>(), w, &la));
            done = true;
          }
        }
        if constexpr (std::is_same<TI, float>::value) {
          if (!unblocked_iface) {
            const bool la = use_lookahead;
            SLAB_TRY(biglu_blocked<TI>(s, Sj, nI, nI, ifPiv.as<int>() + (long long)nI * j, ifInfo.as<int>(),
                                       ifWork.as<TI>(), ifBlkLinv.as<TI>(), panel_kind, la ? side : nullptr,
                                       la ? la_fork : nullptr, la ? la_join : nullptr,
                                       la ? laPerm.as<int>() : nullptr, ifGath.as<int>()));
            done = true;
          }
        }
        if (!done)
          SLAB_TRY(biglu<TI>(s, Sj, nI, nI, ifPiv.as<int>() + (long long)nI * j, ifInfo.as<int>(), ifWork.as<TI>(),
                             panel_kind));
        SLAB_TRY(build_perm(s, ifPiv.as<int>() + (long long)nI * j, nI, ifPerm.as<int>() + (long long)nI * j));
        SLAB_TRY(tri_inv_blocks<TI>(s, Sj, nI, nI, kInvBs, linv(j), uinv(j)));
        if constexpr (std::is_same<TI, double>::value) {
          if (use_emu && use_outer_inv && j + 1 < nbI)
            SLAB_TRY(outer_tri_inverses(s, Sj, nI, nI, linv(j), uinv(j), loinv(j), uoinv(j), emuT.as<double>()));
        }
      }
      SLAB_TRY(split_solve_copies());
    }
    return SLAB_OK;
  }

  // Z = S_j^{-1} F (or S_j^{-T} F) with the stored interface factors: one
  // thread-block cluster for up to eight columns, else the cooperative or the
  // blocked solve.
  int iface_solve(int j, const T* F, T* Z, int nrhs, bool trans) {
    const T* LUj = luS(j);
    const int* pj = ifPerm.as<int>() + (long long)nI * j;
    if (nrhs <= kCoopMaxRhs && kInvBs == kClBs && use_cluster_solve) {
      const int st = trsv_cluster<T>(s, LUj, nI, nI, pj, linvS(j), uinvS(j), F, nI, Z, nI, nrhs, trans);
      if (st != SLAB_ERR_ARG) return st;  // SLAB_ERR_ARG: shape refused before any launch
    }
    if (nrhs <= kCoopMaxRhs) return trsv_coop<T>(s, LUj, nI, nI, pj, linvS(j), uinvS(j), kInvBs, F, nI, Z, nI, nrhs, trans);
    if (trans) return set_error(SLAB_ERR_ARG, "interface: transposed solve takes at most %d columns", kCoopMaxRhs);
    return bigtrs_inv<T>(s, LUj, nI, nI, pj, linvS(j), uinvS(j), kInvBs, F, nI, Z, nI, nrhs);
  }

  int factor_check() {
    // breakdown report
    std::vector<int> hinfo((size_t)nleaf);
    SLAB_CUDA_TRY(cudaMemcpyAsync(hinfo.data(), leafinfo.p, leafinfo.bytes, cudaMemcpyDeviceToHost, s));
    std::vector<int> minfo(mergeinfo.bytes / sizeof(int));
    SLAB_CUDA_TRY(cudaMemcpyAsync(minfo.data(), mergeinfo.p, mergeinfo.bytes, cudaMemcpyDeviceToHost, s));
    int iinfo = 0, eerr = 0;
    if (nbI > 0) SLAB_CUDA_TRY(cudaMemcpyAsync(&iinfo, ifInfo.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (nbI > 0 && use_emu) SLAB_CUDA_TRY(cudaMemcpyAsync(&eerr, emuErr.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    int terr = 0;
    if (use_tc_tree) SLAB_CUDA_TRY(cudaMemcpyAsync(&terr, tcErr.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    SLAB_CUDA_TRY(cudaStreamSynchronize(s));
    tms[0] = elapsed(0, 1);
    tms[1] = elapsed(1, 2);
    tms[2] = elapsed(2, 3);
    factored = true;
    for (size_t i = 0; i < hinfo.size(); ++i)
      if (hinfo[i] > 0) {
        set_error(hinfo[i], "leaf %zu: zero pivot at column %d", i, hinfo[i]);
        return hinfo[i];
      }
    for (size_t i = 0; i < minfo.size(); ++i)
      if (minfo[i] > 0) {
        set_error(minfo[i], "merge %zu: zero pivot at column %d", i, minfo[i]);
        return minfo[i];
      }
    if (iinfo > 0) {
      set_error(iinfo, "interface block: zero pivot at column %d", iinfo);
      return iinfo;
    }
    if (eerr != 0) return set_error(SLAB_ERR_CUDA, "interface: tensor-core pipeline wait expired (code %d)", eerr);
    if (terr != 0) return set_error(SLAB_ERR_CUDA, "merge tree: tensor-core pipeline wait expired (code %d)", terr);
    return SLAB_OK;
  }

  LeafCoeffs coeffs() const {
    return LeafCoeffs{has[0] ? coef[0].as<double>() : nullptr, has[1] ? coef[1].as<double>() : nullptr,
                      has[2] ? coef[2].as<double>() : nullptr, has[3] ? coef[3].as<double>() : nullptr,
                      has[4] ? coef[4].as<double>() : nullptr, has[5] ? coef[5].as<double>() : nullptr};
  }

  int reserve(int nrhs) {
    if (nrhs <= cap_nrhs) return SLAB_OK;
    if (gapp) {
      cudaGraphExecDestroy(gapp);
      gapp = nullptr;
    }
    if (gapp_t) {
      cudaGraphExecDestroy(gapp_t);
      gapp_t = nullptr;
    }
    long long ymax = 0, zmax = 0;
    for (auto& b : batches) {
      b->offY0 = ymax;
      ymax += (long long)b->count * b->nE * nrhs;
      zmax = std::max(zmax, (long long)b->count * b->nO * nrhs);
    }
    SLAB_TRY(wc.alloc((size_t)nleaf * n * nrhs * sizeof(T)));
    SLAB_TRY(flux.alloc((size_t)nleaf * nx * nrhs * sizeof(T)));
    SLAB_TRY(gvec.alloc((size_t)ntot * nrhs * sizeof(T)));
    SLAB_TRY(uvec.alloc((size_t)ntot * nrhs * sizeof(T)));
    SLAB_TRY(Ybuf.alloc((size_t)std::max<long long>(ymax, 1) * sizeof(T)));
    SLAB_TRY(Zbuf.alloc((size_t)std::max<long long>(zmax, (long long)nleaf * nx * nrhs) * sizeof(T)));
    if (nbI > 0) {
      SLAB_TRY(ifF.alloc((size_t)nbI * nI * nrhs * sizeof(T)));
      SLAB_TRY(ifZ.alloc((size_t)nbI * nI * nrhs * sizeof(T)));
    }
    SLAB_TRY(ux_d.alloc((size_t)ntot * nrhs * sizeof(double)));
    SLAB_TRY(uc_d.alloc((size_t)nleaf * n * nrhs * sizeof(double)));
    SLAB_TRY(rc_d.alloc((size_t)nleaf * n * nrhs * sizeof(double)));
    SLAB_TRY(rx_d.alloc((size_t)ntot * nrhs * sizeof(double)));
    SLAB_TRY(rcT.alloc((size_t)nleaf * n * nrhs * sizeof(T)));
    cap_nrhs = nrhs;
    ++epoch_;
    return SLAB_OK;
  }

  // One application of the factorization: input rcT (interior residual,
  // leaf-major) and gvec (face residual); output uvec (face correction) and
  // wc (interior correction, leaf-major).
  int apply(int nrhs) {
    T* g = gvec.as<T>();
    T* u = uvec.as<T>();
    T* w = wc.as<T>();
    const long long strideG = leaf_stride;
    SLAB_CUDA_TRY(cudaMemcpyAsync(w, rcT.p, (size_t)nleaf * n * nrhs * sizeof(T), cudaMemcpyDeviceToDevice, s));
    if (nrhs <= 4 && n <= 32 * kWarpSlots)
      SLAB_TRY(getrs_small<T>(s, n, nrhs, G.as<T>(), nullptr, strideG, n, leafperm.as<int>(), nullptr, n, w, nullptr,
                              (long long)n * nrhs, n, (int)nleaf));
    else if (getrs_many_fits<T>(n))
      SLAB_TRY(getrs_many<T>(s, n, nrhs, G.as<T>(), strideG, n, leafperm.as<int>(), n, w, (long long)n * nrhs, n,
                             (int)nleaf));
    else
      SLAB_TRY(getrs_batched<T>(s, n, nrhs, G.as<T>(), nullptr, strideG, n, piv.as<int>(), nullptr, n, w, nullptr,
                                (long long)n * nrhs, n, (int)nleaf));
    SLAB_TRY(gemm<T>(s, nx, nrhs, n, T(1), NxcT.as<T>(), nullptr, 0, nx, w, nullptr, (long long)n * nrhs, n, T(0),
                     flux.as<T>(), nullptr, (long long)nx * nrhs, nx, (int)nleaf));
    scatter_add_kernel<T><<<grid_for(nleaf * nx * nrhs), 256, 0, s>>>(g, ntot, leafglob.as<int>(), nx, (int)nleaf,
                                                                     nrhs, flux.as<T>(), T(-1), dirmask.as<unsigned char>());
    SLAB_CHECK_LAUNCH();
    // tree forward
    for (auto& bp : batches) {
      Batch& b = *bp;
      T* Y = Ybuf.as<T>() + b.offY0;
      T* Z = Zbuf.as<T>();
      const long long strideM = (long long)b.nE * (b.nE + b.nO);
      T* Maug = fpool.as<T>() + b.offM0;
      gather_kernel<T><<<grid_for((long long)b.count * b.nE * nrhs), 256, 0, s>>>(g, ntot, b.Eglob.as<int>(), b.nE,
                                                                                b.count, nrhs, Y);
      SLAB_CHECK_LAUNCH();
      if (nrhs <= 4 && b.nE <= 32 * kWarpSlots)
        SLAB_TRY(getrs_small<T>(s, b.nE, nrhs, Maug, nullptr, strideM, b.nE, permpool.as<int>() + b.offPiv0,
                                nullptr, b.nE, Y, nullptr, (long long)b.nE * nrhs, b.nE, b.count));
      else if (getrs_many_fits<T>(b.nE))
        SLAB_TRY(getrs_many<T>(s, b.nE, nrhs, Maug, strideM, b.nE, permpool.as<int>() + b.offPiv0, b.nE, Y,
                               (long long)b.nE * nrhs, b.nE, b.count));
      else
        SLAB_TRY(getrs_batched<T>(s, b.nE, nrhs, Maug, nullptr, strideM, b.nE, pivpool.as<int>() + b.offPiv0,
                                  nullptr, b.nE, Y, nullptr, (long long)b.nE * nrhs, b.nE, b.count));
      SLAB_TRY(gemm<T>(s, b.nO, nrhs, b.nE, T(1), fpool.as<T>() + b.offC0, nullptr, (long long)b.nO * b.nE, b.nO, Y,
                       nullptr, (long long)b.nE * nrhs, b.nE, T(0), Z, nullptr, (long long)b.nO * nrhs, b.nO,
                       b.count));
      scatter_add_kernel<T><<<grid_for((long long)b.count * b.nO * nrhs), 256, 0, s>>>(
          g, ntot, b.Oglob.as<int>(), b.nO, b.count, nrhs, Z, T(-1), nullptr);
      SLAB_CHECK_LAUNCH();
    }
    SLAB_CUDA_TRY(cudaMemsetAsync(u, 0, (size_t)ntot * nrhs * sizeof(T), s));
    // interface sweep
    if (nbI > 0) {
      const long long blk = (long long)nI * nI;
      const long long vb = (long long)nI * nrhs;
      T* F = ifF.as<T>();
      T* Zi = ifZ.as<T>();
      gather_kernel<T><<<grid_for((long long)nbI * vb), 256, 0, s>>>(g, ntot, ifGlob.as<int>(), nI, nbI, nrhs, F);
      SLAB_CHECK_LAUNCH();
      for (int j = 0; j < nbI; ++j) {
        if (j > 0)
          SLAB_TRY(gemm<T>(s, nI, nrhs, nI, T(-1), subS(j), nullptr, 0, nI, Zi + vb * (j - 1), nullptr, 0, nI, T(1),
                           F + vb * j, nullptr, 0, nI, 1));
        SLAB_TRY(iface_solve(j, F + vb * j, Zi + vb * j, nrhs, false));
      }
      for (int j = nbI - 2; j >= 0; --j)
        SLAB_TRY(gemm<T>(s, nI, nrhs, nI, T(-1), xS(j), nullptr, 0, nI, Zi + vb * (j + 1), nullptr, 0, nI, T(1),
                         Zi + vb * j, nullptr, 0, nI, 1));
      scatter_set_kernel<T><<<grid_for((long long)nbI * vb), 256, 0, s>>>(u, ntot, ifGlob.as<int>(), nI, nbI, nrhs,
                                                                         Zi);
      SLAB_CHECK_LAUNCH();
    }
    // tree backward
    for (auto it = batches.rbegin(); it != batches.rend(); ++it) {
      Batch& b = **it;
      T* Y = Ybuf.as<T>() + b.offY0;
      T* Z = Zbuf.as<T>();
      const long long strideM = (long long)b.nE * (b.nE + b.nO);
      T* Maug = fpool.as<T>() + b.offM0;
      gather_kernel<T><<<grid_for((long long)b.count * b.nO * nrhs), 256, 0, s>>>(u, ntot, b.Oglob.as<int>(), b.nO,
                                                                                b.count, nrhs, Z);
      SLAB_CHECK_LAUNCH();
      SLAB_TRY(gemm<T>(s, b.nE, nrhs, b.nO, T(-1), Maug + (long long)b.nE * b.nE, nullptr, strideM, b.nE, Z, nullptr,
                       (long long)b.nO * nrhs, b.nO, T(1), Y, nullptr, (long long)b.nE * nrhs, b.nE, b.count));
      scatter_set_kernel<T><<<grid_for((long long)b.count * b.nE * nrhs), 256, 0, s>>>(u, ntot, b.Eglob.as<int>(),
                                                                                     b.nE, b.count, nrhs, Y);
      SLAB_CHECK_LAUNCH();
    }
    // leaf backward: w += S u_x
    gather_kernel<T><<<grid_for(nleaf * nx * nrhs), 256, 0, s>>>(u, ntot, leafglob.as<int>(), nx, (int)nleaf, nrhs,
                                                                flux.as<T>());
    SLAB_CHECK_LAUNCH();
    SLAB_TRY(gemm<T>(s, n, nrhs, nx, T(1), G.as<T>() + (long long)n * n, nullptr, strideG, n, flux.as<T>(), nullptr,
                     (long long)nx * nrhs, nx, T(1), w, nullptr, (long long)n * nrhs, n, (int)nleaf));
    return SLAB_OK;
  }

  // One application of the transposed factorization, nrhs <= 4: input rcT
  // (interior, leaf-major) and gvec (faces, zero on Dirichlet faces); output
  // uvec (face multipliers) and wc (interior multipliers, leaf-major).  Each
  // step is the transpose of a step of apply(), taken in reverse order:
  //   K^T = [A_cc^T  N_c^T; A_cx^T  N_x^T]  ->  DtN^T lam_x = g_x + S^T g_c,
  //   lam_c = A_cc^{-T} (g_c - N_c^T lam_x).
  int apply_t(int nrhs) {
    T* g = gvec.as<T>();
    T* u = uvec.as<T>();
    T* w = wc.as<T>();
    const long long strideG = leaf_stride;
    // leaf forward: g_x += S^T g_c
    SLAB_TRY(gemm_tn<T>(s, nx, nrhs, n, T(1), G.as<T>() + (long long)n * n, nullptr, strideG, n, rcT.as<T>(), nullptr,
                        (long long)n * nrhs, n, T(0), flux.as<T>(), nullptr, (long long)nx * nrhs, nx, (int)nleaf));
    scatter_add_kernel<T><<<grid_for(nleaf * nx * nrhs), 256, 0, s>>>(g, ntot, leafglob.as<int>(), nx, (int)nleaf,
                                                                     nrhs, flux.as<T>(), T(1), dirmask.as<unsigned char>());
    SLAB_CHECK_LAUNCH();
    // tree forward (transposed): g_O -= W^T g_E with W = M^{-1} row; g_E kept in Y
    for (auto& bp : batches) {
      Batch& b = *bp;
      T* Y = Ybuf.as<T>() + b.offY0;
      T* Z = Zbuf.as<T>();
      const long long strideM = (long long)b.nE * (b.nE + b.nO);
      T* Maug = fpool.as<T>() + b.offM0;
      gather_kernel<T><<<grid_for((long long)b.count * b.nE * nrhs), 256, 0, s>>>(g, ntot, b.Eglob.as<int>(), b.nE,
                                                                                b.count, nrhs, Y);
      SLAB_CHECK_LAUNCH();
      SLAB_TRY(gemm_tn<T>(s, b.nO, nrhs, b.nE, T(1), Maug + (long long)b.nE * b.nE, nullptr, strideM, b.nE, Y, nullptr,
                          (long long)b.nE * nrhs, b.nE, T(0), Z, nullptr, (long long)b.nO * nrhs, b.nO, b.count));
      scatter_add_kernel<T><<<grid_for((long long)b.count * b.nO * nrhs), 256, 0, s>>>(
          g, ntot, b.Oglob.as<int>(), b.nO, b.count, nrhs, Z, T(-1), nullptr);
      SLAB_CHECK_LAUNCH();
    }
    SLAB_CUDA_TRY(cudaMemsetAsync(u, 0, (size_t)ntot * nrhs * sizeof(T), s));
    // interface: T = L U with L = [S_j on the diagonal, sub_j below], U = [I, X_j above];
    // T^T x = f: y_j = f_j - X_{j-1}^T y_{j-1}, then x_j = S_j^{-T} (y_j - sub_{j+1}^T x_{j+1})
    if (nbI > 0) {
      const long long blk = (long long)nI * nI;
      const long long vb = (long long)nI * nrhs;
      T* F = ifF.as<T>();
      T* Zi = ifZ.as<T>();
      gather_kernel<T><<<grid_for((long long)nbI * vb), 256, 0, s>>>(g, ntot, ifGlob.as<int>(), nI, nbI, nrhs, F);
      SLAB_CHECK_LAUNCH();
      for (int j = 1; j < nbI; ++j)
        SLAB_TRY(gemm_tn<T>(s, nI, nrhs, nI, T(-1), xS(j - 1), nullptr, 0, nI, F + vb * (j - 1), nullptr, 0, nI, T(1),
                            F + vb * j, nullptr, 0, nI, 1));
      for (int j = nbI - 1; j >= 0; --j) {
        if (j < nbI - 1)
          SLAB_TRY(gemm_tn<T>(s, nI, nrhs, nI, T(-1), subS(j + 1), nullptr, 0, nI, Zi + vb * (j + 1), nullptr, 0, nI,
                              T(1), F + vb * j, nullptr, 0, nI, 1));
        SLAB_TRY(iface_solve(j, F + vb * j, Zi + vb * j, nrhs, true));
      }
      scatter_set_kernel<T><<<grid_for((long long)nbI * vb), 256, 0, s>>>(u, ntot, ifGlob.as<int>(), nI, nbI, nrhs,
                                                                         Zi);
      SLAB_CHECK_LAUNCH();
    }
    // tree backward (transposed): lam_E = M^{-T} (g_E - col^T lam_O)
    for (auto it = batches.rbegin(); it != batches.rend(); ++it) {
      Batch& b = **it;
      T* Y = Ybuf.as<T>() + b.offY0;
      T* Z = Zbuf.as<T>();
      const long long strideM = (long long)b.nE * (b.nE + b.nO);
      T* Maug = fpool.as<T>() + b.offM0;
      gather_kernel<T><<<grid_for((long long)b.count * b.nO * nrhs), 256, 0, s>>>(u, ntot, b.Oglob.as<int>(), b.nO,
                                                                                b.count, nrhs, Z);
      SLAB_CHECK_LAUNCH();
      SLAB_TRY(gemm_tn<T>(s, b.nE, nrhs, b.nO, T(-1), fpool.as<T>() + b.offC0, nullptr, (long long)b.nO * b.nE, b.nO,
                          Z, nullptr, (long long)b.nO * nrhs, b.nO, T(1), Y, nullptr, (long long)b.nE * nrhs, b.nE,
                          b.count));
      SLAB_TRY(getrs_small_t<T>(s, b.nE, nrhs, Maug, nullptr, strideM, b.nE, permpool.as<int>() + b.offPiv0, nullptr,
                                b.nE, Y, nullptr, (long long)b.nE * nrhs, b.nE, b.count));
      scatter_set_kernel<T><<<grid_for((long long)b.count * b.nE * nrhs), 256, 0, s>>>(u, ntot, b.Eglob.as<int>(),
                                                                                     b.nE, b.count, nrhs, Y);
      SLAB_CHECK_LAUNCH();
    }
    // leaf backward: lam_c = A_cc^{-T} (g_c - N_c^T lam_x)
    gather_kernel<T><<<grid_for(nleaf * nx * nrhs), 256, 0, s>>>(u, ntot, leafglob.as<int>(), nx, (int)nleaf, nrhs,
                                                                flux.as<T>());
    SLAB_CHECK_LAUNCH();
    SLAB_CUDA_TRY(cudaMemcpyAsync(w, rcT.p, (size_t)nleaf * n * nrhs * sizeof(T), cudaMemcpyDeviceToDevice, s));
    SLAB_TRY(gemm_tn<T>(s, n, nrhs, nx, T(-1), NxcT.as<T>(), nullptr, 0, nx, flux.as<T>(), nullptr,
                        (long long)nx * nrhs, nx, T(1), w, nullptr, (long long)n * nrhs, n, (int)nleaf));
    return getrs_small_t<T>(s, n, nrhs, G.as<T>(), nullptr, strideG, n, leafperm.as<int>(), nullptr, n, w, nullptr,
                            (long long)n * nrhs, n, (int)nleaf);
  }

  int residual_t_impl(int nrhs, const double* lx, const double* lc, const double* gint, const double* gfaces,
                      double* rc, double* rx, bool all_faces) {
    mask_faces_kernel<<<grid_for(ntot * nrhs), 256, 0, s>>>(gfaces, dirmask.as<unsigned char>(), rx, ntot, nrhs, 0);
    SLAB_CHECK_LAUNCH();
    if (all_faces) {
      // Dirichlet columns start from the direct sensitivity as well
      SLAB_CUDA_TRY(cudaMemcpyAsync(rx, gfaces, (size_t)ntot * nrhs * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
    ResidualArgs r{};
    r.p = p; r.q = q; r.n = n; r.nx = nx; r.nleaf = (int)nleaf; r.nrhs = nrhs; r.ntot = ntot;
    r.co = coeffs(); r.D = D.as<double>(); r.Dsq = Dsq.as<double>();
    r.leafglob = leafglob.as<int>(); r.dirmask = dirmask.as<unsigned char>();
    r.ux = lx; r.uc = lc; r.fbody = gint; r.rc = rc; r.rx = rx; r.all_faces = all_faces ? 1 : 0;
    if (mixed) {
      r.interp = interp.as<double>(); r.jxr = jxr.as<int>(); r.nxa = 4 * (p - 1);
      const size_t bytes = (9 * (size_t)p * p + nx) * sizeof(double);
      SLAB_TRY(ensure_smem(residual_t_mixed_kernel, bytes, "residual_t_mixed"));
      residual_t_mixed_kernel<<<(unsigned)nleaf, 256, bytes, s>>>(r);
    } else {
      residual_t_kernel<<<(unsigned)nleaf, 256, (6 * (size_t)p * p + nx) * sizeof(double), s>>>(r);
    }
    SLAB_CHECK_LAUNCH();
    return SLAB_OK;
  }

  int reserve_t(int nrhs) {
    SLAB_TRY(reserve(nrhs));
    if (gi_d.bytes < (size_t)nleaf * n * nrhs * sizeof(double)) {
      SLAB_TRY(gi_d.alloc((size_t)nleaf * n * nrhs * sizeof(double)));
      SLAB_TRY(gf_d.alloc((size_t)ntot * nrhs * sizeof(double)));
    }
    return SLAB_OK;
  }

  int adjoint(int nrhs, const double* gleaf, const double* gfaces, double tol, int max_iter, double* lam_leaf,
              double* lam_faces, double* gbnd, int* iters, double* stats) override {
    SLAB_TRY(enter());
    int st = SLAB_OK, total_it = 0;
    double worst[5] = {0, 0, 0, 0, 0};
    const long long npts = nleaf * p * p;
    // the transposed solve kernels take up to four right-hand sides at a time
    for (int c0 = 0; c0 < nrhs && (st == SLAB_OK || st == SLAB_ERR_NOCONV); c0 += 4) {
      const int k = std::min(4, nrhs - c0);
      int it = 0;
      double sv[5] = {0, 0, 0, 0, 0};
      const int sc = adjoint_impl(k, gleaf ? gleaf + c0 * npts : nullptr, gfaces ? gfaces + c0 * ntot : nullptr, tol,
                                  max_iter, lam_leaf ? lam_leaf + c0 * npts : nullptr,
                                  lam_faces ? lam_faces + c0 * ntot : nullptr, gbnd ? gbnd + c0 * ntot : nullptr, &it,
                                  sv);
      if (sc != SLAB_OK && st == SLAB_OK) st = sc;
      total_it = std::max(total_it, it);
      for (int i = 0; i < 5; ++i) worst[i] = std::max(worst[i], sv[i]);
      if (sc != SLAB_OK && sc != SLAB_ERR_NOCONV) break;
    }
    if (iters) *iters = total_it;
    if (stats)
      for (int i = 0; i < 5; ++i) stats[i] = worst[i];
    const int st2 = leave();
    if (st == SLAB_ERR_NOCONV) set_error(SLAB_ERR_NOCONV, "adjoint refinement did not reach tol %.1e", tol);
    return st != SLAB_OK ? st : st2;
  }

  int adjoint_impl(int nrhs, const double* gleaf, const double* gfaces, double tol, int max_iter, double* lam_leaf,
                   double* lam_faces, double* gbnd, int* iters, double* stats) {
    if (!factored) return set_error(SLAB_ERR_STATE, "slab_engine_adjoint: engine not factored");
    if (nrhs <= 0 || (!gleaf && !gfaces)) return set_error(SLAB_ERR_ARG, "slab_engine_adjoint: invalid arguments");
    if (n > 32 * kWarpSlots) return set_error(SLAB_ERR_ARG, "slab_engine_adjoint: leaf order p=%d too large", p);
    for (auto& b : batches)
      if (b->nE > 32 * kWarpSlots)
        return set_error(SLAB_ERR_ARG, "slab_engine_adjoint: merge block of order %d > %d", b->nE, 32 * kWarpSlots);
    SLAB_TRY(reserve_t(nrhs));
    const long long nc_el = nleaf * n * nrhs, nf_el = ntot * nrhs;
    double* gi = gi_d.as<double>();
    double* gf = gf_d.as<double>();
    if (gfaces)
      SLAB_CUDA_TRY(cudaMemcpyAsync(gf, gfaces, (size_t)nf_el * sizeof(double), cudaMemcpyDeviceToDevice, s));
    else
      SLAB_CUDA_TRY(cudaMemsetAsync(gf, 0, (size_t)nf_el * sizeof(double), s));
    if (gleaf) {
      AssembleTArgs at{};
      at.p = p; at.q = q; at.n = n; at.nx = nx; at.nleaf = (int)nleaf; at.nrhs = nrhs; at.ntot = ntot;
      at.leafglob = leafglob.as<int>(); at.interp = interp.as<double>(); at.jxreorder = jxr.as<int>();
      at.dsol = gleaf; at.gint = gi; at.gfaces = gf;
      assemble_t_kernel<<<(unsigned)nleaf, 256, 0, s>>>(at);
      SLAB_CHECK_LAUNCH();
    } else {
      SLAB_CUDA_TRY(cudaMemsetAsync(gi, 0, (size_t)nc_el * sizeof(double), s));
    }
    SLAB_CUDA_TRY(cudaMemsetAsync(uc_d.p, 0, (size_t)nc_el * sizeof(double), s));
    SLAB_CUDA_TRY(cudaMemsetAsync(ux_d.p, 0, (size_t)nf_el * sizeof(double), s));
    double r0 = 0, rn = 0, rel = 1.0, dn = 0, un = 0;
    int it = 0;
    bool converged = false;
    for (; it < max_iter; ++it) {
      SLAB_TRY(residual_t_impl(nrhs, ux_d.as<double>(), uc_d.as<double>(), gi, gf, rc_d.as<double>(),
                               rx_d.as<double>(), false));
      SLAB_TRY(norms(rc_d.p, true, nc_el, rx_d.p, true, nf_el, &rn));
      if (it == 0) r0 = rn;
      if (rn == 0.0) {
        converged = true;
        rel = 0.0;
        break;
      }
      convert_kernel<T, double><<<grid_for(nc_el), 256, 0, s>>>(rc_d.as<double>(), rcT.as<T>(), nc_el);
      SLAB_CHECK_LAUNCH();
      convert_kernel<T, double><<<grid_for(nf_el), 256, 0, s>>>(rx_d.as<double>(), gvec.as<T>(), nf_el);
      SLAB_CHECK_LAUNCH();
      if (gapp_t && gapp_t_nrhs != nrhs) {
        cudaGraphExecDestroy(gapp_t);
        gapp_t = nullptr;
      }
      gapp_t_nrhs = nrhs;
      SLAB_TRY(run_graph(gapp_t, [&]() { return apply_t(nrhs); }));
      axpy_kernel<T><<<grid_for(nc_el), 256, 0, s>>>(uc_d.as<double>(), wc.as<T>(), nc_el);
      SLAB_CHECK_LAUNCH();
      axpy_kernel<T><<<grid_for(nf_el), 256, 0, s>>>(ux_d.as<double>(), uvec.as<T>(), nf_el);
      SLAB_CHECK_LAUNCH();
      SLAB_TRY(norms(wc.p, false, nc_el, uvec.p, false, nf_el, &dn));
      SLAB_TRY(norms(uc_d.p, true, nc_el, ux_d.p, true, nf_el, &un));
      rel = un > 0 ? dn / un : 0.0;
      if (rel <= tol) {
        converged = true;
        ++it;
        break;
      }
    }
    // final transposed residual over every face column: the Dirichlet entries
    // are the sensitivity of the loss to the Dirichlet data
    SLAB_TRY(residual_t_impl(nrhs, ux_d.as<double>(), uc_d.as<double>(), gi, gf, rc_d.as<double>(), rx_d.as<double>(),
                             true));
    SLAB_TRY(norms(rc_d.p, true, nc_el, nullptr, true, 0, &rn));
    if (gbnd) {
      mask_faces_kernel<<<grid_for(nf_el), 256, 0, s>>>(rx_d.as<double>(), dirmask.as<unsigned char>(), gbnd, ntot,
                                                        nrhs, 1);
      SLAB_CHECK_LAUNCH();
    }
    // residual over the unknown rows only, for the report
    mask_faces_kernel<<<grid_for(nf_el), 256, 0, s>>>(rx_d.as<double>(), dirmask.as<unsigned char>(),
                                                      rx_d.as<double>(), ntot, nrhs, 0);
    SLAB_CHECK_LAUNCH();
    SLAB_TRY(norms(rc_d.p, true, nc_el, rx_d.p, true, nf_el, &rn));
    if (lam_faces)
      SLAB_CUDA_TRY(cudaMemcpyAsync(lam_faces, ux_d.p, (size_t)nf_el * sizeof(double), cudaMemcpyDeviceToDevice, s));
    if (lam_leaf) {
      interior_to_nodes_kernel<<<grid_for(nleaf * p * p * nrhs), 256, 0, s>>>(uc_d.as<double>(), lam_leaf, p,
                                                                             (int)nleaf, nrhs);
      SLAB_CHECK_LAUNCH();
    }
    SLAB_CUDA_TRY(cudaStreamSynchronize(s));
    if (iters) *iters = it;
    if (stats) {
      stats[0] = rel;
      stats[1] = rn;
      stats[2] = r0;
      stats[3] = 0.0;
      stats[4] = r0 > 0 ? rn / r0 : 0.0;
    }
    if (!converged) {
      set_error(SLAB_ERR_NOCONV, "adjoint refinement: relative correction %.3e after %d steps (tol %.1e)", rel, it,
                tol);
      return SLAB_ERR_NOCONV;
    }
    return SLAB_OK;
  }

  int coeff_grad(int nrhs, const double* ufaces, const double* uleaf, const double* lam_leaf, double* g11,
                 double* g22, double* g12, double* g1, double* g2, double* g0) override {
    if (g12 && !mixed)
      return set_error(SLAB_ERR_ARG, "slab_engine_coeff_grad_mixed: the engine has no mixed derivative (c12)");
    if (nrhs <= 0 || !ufaces || !uleaf || !lam_leaf)
      return set_error(SLAB_ERR_ARG, "slab_engine_coeff_grad: invalid arguments");
    if (n > 4 * 256) return set_error(SLAB_ERR_ARG, "slab_engine_coeff_grad: leaf order p=%d too large", p);
    SLAB_TRY(enter());
    GradArgs ga{};
    ga.p = p; ga.q = q; ga.n = n; ga.nx = nx; ga.nleaf = (int)nleaf; ga.nrhs = nrhs; ga.ntot = ntot;
    ga.D = D.as<double>(); ga.Dsq = Dsq.as<double>(); ga.leafglob = leafglob.as<int>();
    ga.uleaf = uleaf; ga.ufaces = ufaces; ga.lam = lam_leaf;
    ga.g11 = g11; ga.g22 = g22; ga.g1 = g1; ga.g2 = g2; ga.g0 = g0;
    if (mixed) {
      ga.g12 = g12; ga.interp = interp.as<double>(); ga.jxr = jxr.as<int>(); ga.nxa = 4 * (p - 1);
      const size_t bytes = (4 * (size_t)p * p + nx) * sizeof(double);
      SLAB_TRY(ensure_smem(coeff_grad_mixed_kernel, bytes, "coeff_grad_mixed"));
      coeff_grad_mixed_kernel<<<(unsigned)nleaf, 256, bytes, s>>>(ga);
    } else {
      coeff_grad_kernel<<<(unsigned)nleaf, 256, 3 * (size_t)p * p * sizeof(double), s>>>(ga);
    }
    SLAB_CHECK_LAUNCH();
    return leave();
  }

  int residual_impl(int nrhs, const double* ux, const double* uc, const double* fbody, double* rc, double* rx) {
    SLAB_CUDA_TRY(cudaMemsetAsync(rx, 0, (size_t)ntot * nrhs * sizeof(double), s));
    ResidualArgs r{};
    r.p = p; r.q = q; r.n = n; r.nx = nx; r.nleaf = (int)nleaf; r.nrhs = nrhs; r.ntot = ntot;
    r.co = coeffs(); r.D = D.as<double>(); r.Dsq = Dsq.as<double>();
    r.leafglob = leafglob.as<int>(); r.dirmask = dirmask.as<unsigned char>();
    r.ux = ux; r.uc = uc; r.fbody = fbody; r.rc = rc; r.rx = rx;
    if (mixed) {
      r.interp = interp.as<double>(); r.jxr = jxr.as<int>(); r.nxa = 4 * (p - 1);
      const size_t bytes = (4 * (size_t)p * p + nx) * sizeof(double);
      SLAB_TRY(ensure_smem(residual_mixed_kernel, bytes, "residual_mixed"));
      residual_mixed_kernel<<<(unsigned)nleaf, 256, bytes, s>>>(r);
    } else {
      residual_kernel<<<(unsigned)nleaf, 256, 3 * (size_t)p * p * sizeof(double), s>>>(r);
    }
    SLAB_CHECK_LAUNCH();
    return SLAB_OK;
  }

  int norms(const void* x1, bool x1d, long long n1_, const void* x2, bool x2d, long long n2_, double* out) {
    SLAB_CUDA_TRY(cudaMemsetAsync(acc.p, 0, sizeof(double), s));
    if (n1_ > 0) {
      if (x1d)
        sumsq_kernel<double><<<grid_for(n1_), 256, 0, s>>>((const double*)x1, n1_, acc.as<double>());
      else
        sumsq_kernel<T><<<grid_for(n1_), 256, 0, s>>>((const T*)x1, n1_, acc.as<double>());
      SLAB_CHECK_LAUNCH();
    }
    if (n2_ > 0) {
      if (x2d)
        sumsq_kernel<double><<<grid_for(n2_), 256, 0, s>>>((const double*)x2, n2_, acc.as<double>());
      else
        sumsq_kernel<T><<<grid_for(n2_), 256, 0, s>>>((const T*)x2, n2_, acc.as<double>());
      SLAB_CHECK_LAUNCH();
    }
    double h = 0;
    SLAB_CUDA_TRY(cudaMemcpyAsync(&h, acc.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    SLAB_CUDA_TRY(cudaStreamSynchronize(s));
    *out = std::sqrt(h);
    return SLAB_OK;
  }

  int solve(int nrhs, const double* bnd, const double* fbody, double tol, int max_iter, double* ufaces,
            double* uleaf, int* iters, double* stats) override {
    SLAB_TRY(enter());
    const int st = solve_impl(nrhs, bnd, fbody, tol, max_iter, ufaces, uleaf, iters, stats);
    const int st2 = leave();
    return st != SLAB_OK ? st : st2;
  }

  int solve_impl(int nrhs, const double* bnd, const double* fbody, double tol, int max_iter, double* ufaces,
                 double* uleaf, int* iters, double* stats) {
    if (!factored) return set_error(SLAB_ERR_STATE, "slab_engine_solve: engine not factored");
    if (nrhs <= 0 || !bnd) return set_error(SLAB_ERR_ARG, "slab_engine_solve: invalid arguments");
    SLAB_TRY(reserve(nrhs));
    SLAB_CUDA_TRY(cudaEventRecord(ev[4], s));
    tms[4] = 0.0;
    tms[5] = 0.0;
    const long long nc_el = nleaf * n * nrhs, nf_el = ntot * nrhs;
    init_faces_kernel<<<grid_for(nf_el), 256, 0, s>>>(bnd, dirmask.as<unsigned char>(), ux_d.as<double>(), ntot, nrhs);
    SLAB_CHECK_LAUNCH();
    SLAB_CUDA_TRY(cudaMemsetAsync(uc_d.p, 0, (size_t)nc_el * sizeof(double), s));
    // body load in leaf-major interior layout is read directly by the residual kernel
    double r0 = 0, rn = 0, rel = 1.0, dn = 0, un = 0;
    int it = 0;
    bool converged = false;
    for (; it < max_iter; ++it) {
      SLAB_TRY(residual_impl(nrhs, ux_d.as<double>(), uc_d.as<double>(), fbody, rc_d.as<double>(), rx_d.as<double>()));
      SLAB_TRY(norms(rc_d.p, true, nc_el, rx_d.p, true, nf_el, &rn));
      if (it == 0) r0 = rn;
      if (rn == 0.0) {
        converged = true;
        rel = 0.0;
        break;
      }
      convert_kernel<T, double><<<grid_for(nc_el), 256, 0, s>>>(rc_d.as<double>(), rcT.as<T>(), nc_el);
      SLAB_CHECK_LAUNCH();
      convert_kernel<T, double><<<grid_for(nf_el), 256, 0, s>>>(rx_d.as<double>(), gvec.as<T>(), nf_el);
      SLAB_CHECK_LAUNCH();
      SLAB_CUDA_TRY(cudaEventRecord(ev[6], s));
      if (gapp && gapp_nrhs != nrhs) {
        cudaGraphExecDestroy(gapp);
        gapp = nullptr;
      }
      gapp_nrhs = nrhs;
      SLAB_TRY(run_graph(gapp, [&]() { return apply(nrhs); }));
      SLAB_CUDA_TRY(cudaEventRecord(ev[7], s));
      axpy_kernel<T><<<grid_for(nc_el), 256, 0, s>>>(uc_d.as<double>(), wc.as<T>(), nc_el);
      SLAB_CHECK_LAUNCH();
      axpy_kernel<T><<<grid_for(nf_el), 256, 0, s>>>(ux_d.as<double>(), uvec.as<T>(), nf_el);
      SLAB_CHECK_LAUNCH();
      SLAB_TRY(norms(wc.p, false, nc_el, uvec.p, false, nf_el, &dn));
      tms[4] += elapsed(6, 7);
      tms[5] += 1;
      SLAB_TRY(norms(uc_d.p, true, nc_el, ux_d.p, true, nf_el, &un));
      rel = un > 0 ? dn / un : 0.0;
      if (rel <= tol) {
        converged = true;
        ++it;
        break;
      }
    }
    // final residual and interior-residual norm
    SLAB_TRY(residual_impl(nrhs, ux_d.as<double>(), uc_d.as<double>(), fbody, rc_d.as<double>(), rx_d.as<double>()));
    double rloc = 0;
    SLAB_TRY(norms(rc_d.p, true, nc_el, nullptr, true, 0, &rloc));
    SLAB_TRY(norms(rc_d.p, true, nc_el, rx_d.p, true, nf_el, &rn));
    if (ufaces)
      SLAB_CUDA_TRY(cudaMemcpyAsync(ufaces, ux_d.p, (size_t)nf_el * sizeof(double), cudaMemcpyDeviceToDevice, s));
    if (uleaf) {
      AssembleArgs aa{};
      aa.p = p; aa.q = q; aa.n = n; aa.nx = nx; aa.nleaf = (int)nleaf; aa.nrhs = nrhs; aa.ntot = ntot;
      aa.leafglob = leafglob.as<int>(); aa.interp = interp.as<double>(); aa.jxreorder = jxr.as<int>();
      aa.ispan = ispan.as<int>();
      aa.ux = ux_d.as<double>(); aa.uc = uc_d.as<double>(); aa.out = uleaf;
      assemble_solution_kernel<<<(unsigned)nleaf, 256, (size_t)nx * kAssembleRhs * sizeof(double), s>>>(aa);
      SLAB_CHECK_LAUNCH();
    }
    SLAB_CUDA_TRY(cudaEventRecord(ev[5], s));
    SLAB_CUDA_TRY(cudaEventSynchronize(ev[5]));
    tms[3] = elapsed(4, 5);
    if (iters) *iters = it;
    if (stats) {
      stats[0] = rel;
      stats[1] = rn;
      stats[2] = r0;
      stats[3] = rloc;
      stats[4] = r0 > 0 ? rn / r0 : 0.0;
    }
    SLAB_CUDA_TRY(cudaStreamSynchronize(s));
    if (!converged) {
      set_error(SLAB_ERR_NOCONV, "refinement: relative correction %.3e after %d steps (tol %.1e)", rel, it, tol);
      return SLAB_ERR_NOCONV;
    }
    return SLAB_OK;
  }

  // ---- the refined solve as one CUDA graph --------------------------------------
  // Adds to G: the set-up of a solve, a conditional WHILE node whose body is one
  // refinement step (FP64 residual, application of the factors, update, and a
  // one-thread kernel that decides on the device whether another step runs), and
  // the final residual and assembly into uleaf.  bnd, fbody and uleaf are device
  // buffers of the caller, read and written at every launch of the graph.
  DevBuf gstat;
  long long gr_pre = 0, gr_body = 0, gr_post = 0;
  cudaStream_t stream() const override { return s; }
  long long epoch() const override { return epoch_; }

  int sumsq_into(const void* x, bool xd, long long nel, double* slot) {
    if (nel <= 0) return SLAB_OK;
    if (xd)
      sumsq_kernel<double><<<grid_for(nel), 256, 0, s>>>((const double*)x, nel, slot);
    else
      sumsq_kernel<T><<<grid_for(nel), 256, 0, s>>>((const T*)x, nel, slot);
    SLAB_CHECK_LAUNCH();
    return SLAB_OK;
  }

  int capture_solve(cudaGraph_t G, int nrhs, const double* bnd, const double* fbody, double* uleaf, double tol,
                    int max_iter) override {
    if (!factored) return set_error(SLAB_ERR_STATE, "solve graph: engine not factored");
    if (nrhs <= 0 || !bnd || !uleaf || max_iter <= 0) return set_error(SLAB_ERR_ARG, "solve graph: invalid arguments");
    SLAB_TRY(reserve(nrhs));
    SLAB_TRY(gstat.ensure(kGstatWords * sizeof(double)));
    SLAB_CUDA_TRY(cudaStreamSynchronize(s));
    const long long nc_el = nleaf * n * nrhs, nf_el = ntot * nrhs;
    double* st = gstat.as<double>();
    // set-up: faces with the Dirichlet data, zero interiors and status
    long long c0 = launch_count();
    SLAB_CUDA_TRY(cudaStreamBeginCaptureToGraph(s, G, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    int stc = SLAB_OK;
    {
      init_faces_kernel<<<grid_for(nf_el), 256, 0, s>>>(bnd, dirmask.as<unsigned char>(), ux_d.as<double>(), ntot,
                                                       nrhs);
      count_launch();
      if (cudaMemsetAsync(uc_d.p, 0, (size_t)nc_el * sizeof(double), s) != cudaSuccess ||
          cudaMemsetAsync(st, 0, kGstatWords * sizeof(double), s) != cudaSuccess)
        stc = set_error(SLAB_ERR_CUDA, "solve graph: set-up capture failed");
    }
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    cudaGraph_t cg = nullptr;
    std::vector<cudaGraphNode_t> pre_sinks;
    if (cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, &deps, nullptr, &ndeps) == cudaSuccess)
      pre_sinks.assign(deps, deps + ndeps);
    cudaGraph_t gout = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(s, &gout);
    if (stc != SLAB_OK) return stc;
    if (ee != cudaSuccess) return set_error(SLAB_ERR_CUDA, "solve graph: set-up capture: %s", cudaGetErrorString(ee));
    gr_pre = launch_count() - c0;
    add_launches(-gr_pre);
    // the WHILE node
    cudaGraphConditionalHandle h;
    SLAB_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, G, 1u, cudaGraphCondAssignDefault));
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t cnode;
    SLAB_CUDA_TRY(cudaGraphAddNode(&cnode, G, pre_sinks.data(), nullptr, pre_sinks.size(), &np));
    cudaGraph_t body = np.conditional.phGraph_out[0];
    // one refinement step
    c0 = launch_count();
    SLAB_CUDA_TRY(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    stc = [&]() -> int {
      SLAB_TRY(residual_impl(nrhs, ux_d.as<double>(), uc_d.as<double>(), fbody, rc_d.as<double>(), rx_d.as<double>()));
      SLAB_TRY(sumsq_into(rc_d.p, true, nc_el, st + 1));
      SLAB_TRY(sumsq_into(rx_d.p, true, nf_el, st + 1));
      convert_kernel<T, double><<<grid_for(nc_el), 256, 0, s>>>(rc_d.as<double>(), rcT.as<T>(), nc_el);
      SLAB_CHECK_LAUNCH();
      convert_kernel<T, double><<<grid_for(nf_el), 256, 0, s>>>(rx_d.as<double>(), gvec.as<T>(), nf_el);
      SLAB_CHECK_LAUNCH();
      SLAB_TRY(apply(nrhs));
      axpy_kernel<T><<<grid_for(nc_el), 256, 0, s>>>(uc_d.as<double>(), wc.as<T>(), nc_el);
      SLAB_CHECK_LAUNCH();
      axpy_kernel<T><<<grid_for(nf_el), 256, 0, s>>>(ux_d.as<double>(), uvec.as<T>(), nf_el);
      SLAB_CHECK_LAUNCH();
      SLAB_TRY(sumsq_into(wc.p, false, nc_el, st + 3));
      SLAB_TRY(sumsq_into(uvec.p, false, nf_el, st + 3));
      SLAB_TRY(sumsq_into(uc_d.p, true, nc_el, st + 4));
      SLAB_TRY(sumsq_into(ux_d.p, true, nf_el, st + 4));
      refine_step_kernel<<<1, 32, 0, s>>>(h, st, tol, max_iter);
      SLAB_CHECK_LAUNCH();
      return SLAB_OK;
    }();
    const cudaError_t eb = cudaStreamEndCapture(s, &body);
    if (stc != SLAB_OK) return stc;
    if (eb != cudaSuccess) return set_error(SLAB_ERR_CUDA, "solve graph: step capture: %s", cudaGetErrorString(eb));
    gr_body = launch_count() - c0;
    add_launches(-gr_body);
    // final residual and the leaf-node solution
    c0 = launch_count();
    SLAB_CUDA_TRY(cudaStreamBeginCaptureToGraph(s, G, &cnode, nullptr, 1, cudaStreamCaptureModeRelaxed));
    stc = [&]() -> int {
      SLAB_TRY(residual_impl(nrhs, ux_d.as<double>(), uc_d.as<double>(), fbody, rc_d.as<double>(), rx_d.as<double>()));
      SLAB_TRY(sumsq_into(rc_d.p, true, nc_el, st + 8));
      SLAB_TRY(sumsq_into(rc_d.p, true, nc_el, st + 7));
      SLAB_TRY(sumsq_into(rx_d.p, true, nf_el, st + 7));
      AssembleArgs aa{};
      aa.p = p; aa.q = q; aa.n = n; aa.nx = nx; aa.nleaf = (int)nleaf; aa.nrhs = nrhs; aa.ntot = ntot;
      aa.leafglob = leafglob.as<int>(); aa.interp = interp.as<double>(); aa.jxreorder = jxr.as<int>();
      aa.ispan = ispan.as<int>();
      aa.ux = ux_d.as<double>(); aa.uc = uc_d.as<double>(); aa.out = uleaf;
      assemble_solution_kernel<<<(unsigned)nleaf, 256, (size_t)nx * kAssembleRhs * sizeof(double), s>>>(aa);
      SLAB_CHECK_LAUNCH();
      return SLAB_OK;
    }();
    const cudaError_t ep = cudaStreamEndCapture(s, &gout);
    if (stc != SLAB_OK) return stc;
    if (ep != cudaSuccess) return set_error(SLAB_ERR_CUDA, "solve graph: final capture: %s", cudaGetErrorString(ep));
    gr_post = launch_count() - c0;
    add_launches(-gr_post);
    return SLAB_OK;
  }

  int graph_status(int* iters, double* stats, bool count) override {
    double h[kGstatWords];
    if (!gstat.p) return set_error(SLAB_ERR_STATE, "solve graph: no graph captured on this engine");
    SLAB_CUDA_TRY(cudaMemcpy(h, gstat.p, sizeof(h), cudaMemcpyDeviceToHost));
    const int it = (int)h[0];
    if (count) add_launches(gr_pre + gr_post + gr_body * it);
    if (iters) *iters = it;
    if (stats) {
      const double r0 = std::sqrt(h[2]), rn = std::sqrt(h[7]);
      stats[0] = h[5];
      stats[1] = rn;
      stats[2] = r0;
      stats[3] = std::sqrt(h[8]);
      stats[4] = r0 > 0 ? rn / r0 : 0.0;
    }
    if (h[6] == 0.0)
      return set_error(SLAB_ERR_NOCONV, "refinement (graph): relative correction %.3e after %d steps", h[5], it);
    return SLAB_OK;
  }

  // One application of the factorization to a residual (FP64 in and out, the
  // layouts of residual()): the correction step of the refinement, alone.
  int apply_once(int nrhs, const double* rint, const double* rfaces, double* dint, double* dfaces) override {
    if (!factored) return set_error(SLAB_ERR_STATE, "slab_engine_apply: engine not factored");
    if (nrhs <= 0 || !rint || !rfaces || !dint || !dfaces)
      return set_error(SLAB_ERR_ARG, "slab_engine_apply: invalid arguments");
    SLAB_TRY(enter());
    const int st = apply_once_impl(nrhs, rint, rfaces, dint, dfaces);
    const int st2 = leave();
    return st != SLAB_OK ? st : st2;
  }

  int apply_once_impl(int nrhs, const double* rint, const double* rfaces, double* dint, double* dfaces) {
    SLAB_TRY(reserve(nrhs));
    const long long nc_el = nleaf * n * nrhs, nf_el = ntot * nrhs;
    convert_kernel<T, double><<<grid_for(nc_el), 256, 0, s>>>(rint, rcT.as<T>(), nc_el);
    SLAB_CHECK_LAUNCH();
    // Dirichlet faces carry no flux row: their entries are read as zero
    mask_faces_kernel<<<grid_for(nf_el), 256, 0, s>>>(rfaces, dirmask.as<unsigned char>(), rx_d.as<double>(), ntot,
                                                      nrhs, 0);
    SLAB_CHECK_LAUNCH();
    convert_kernel<T, double><<<grid_for(nf_el), 256, 0, s>>>(rx_d.as<double>(), gvec.as<T>(), nf_el);
    SLAB_CHECK_LAUNCH();
    if (gapp && gapp_nrhs != nrhs) {
      cudaGraphExecDestroy(gapp);
      gapp = nullptr;
    }
    gapp_nrhs = nrhs;
    SLAB_TRY(run_graph(gapp, [&]() { return apply(nrhs); }));
    convert_kernel<double, T><<<grid_for(nc_el), 256, 0, s>>>(wc.as<T>(), dint, nc_el);
    SLAB_CHECK_LAUNCH();
    convert_kernel<double, T><<<grid_for(nf_el), 256, 0, s>>>(uvec.as<T>(), dfaces, nf_el);
    SLAB_CHECK_LAUNCH();
    SLAB_CUDA_TRY(cudaStreamSynchronize(s));
    return SLAB_OK;
  }

  int residual(int nrhs, const double* ufaces, const double* uint, const double* fbody, double* rint,
               double* rfaces) override {
    if (!factored && !has[0] && !has[1] && !has[4])
      return set_error(SLAB_ERR_STATE, "slab_engine_residual: coefficients not set (call factor first)");
    SLAB_TRY(enter());
    SLAB_TRY(residual_impl(nrhs, ufaces, uint, fbody, rint, rfaces));
    SLAB_CUDA_TRY(cudaStreamSynchronize(s));
    return leave();
  }
};

}  // namespace slab

struct slab_engine {
  std::unique_ptr<slab::EngineBase> impl;
};

extern "C" int slab_version(void) { return 100; }

extern "C" const char* slab_last_error(void) { return slab::last_error(); }

static int engine_create(slab_engine** out, int p, int n0, int n1, int buf, int precision, const double* hD,
                         const double* hDsq, const double* hNx, const double* hinterp, const int* hjxr, void* stream,
                         bool mixed) {
  if (!out || p < 4 || n0 < 1 || n1 < 1 || buf < 1 || n0 % buf != 0 || !hD || !hDsq || !hNx || !hinterp || !hjxr)
    return slab::set_error(SLAB_ERR_ARG, "slab_engine_create: invalid geometry or null operator");
  const long long ntot = (long long)(p - 2) * ((long long)n0 * (2 * n1 + 1) + n1);
  if (ntot >= (1LL << 31)) return slab::set_error(SLAB_ERR_ARG, "slab_engine_create: problem too large for int32 indexing");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  auto e = std::make_unique<slab_engine>();
  int st = SLAB_OK;
  if (precision == SLAB_PREC_FP64) {
    auto im = std::make_unique<slab::EngineImpl<double, double>>(p, n0, n1, buf, s, mixed);
    st = im->init(hD, hDsq, hNx, hinterp, hjxr);
    e->impl = std::move(im);
  } else if (precision == SLAB_PREC_MIXED) {
    auto im = std::make_unique<slab::EngineImpl<float, double>>(p, n0, n1, buf, s, mixed);
    st = im->init(hD, hDsq, hNx, hinterp, hjxr);
    e->impl = std::move(im);
  } else if (precision == SLAB_PREC_FP32) {
    auto im = std::make_unique<slab::EngineImpl<float, float>>(p, n0, n1, buf, s, mixed);
    st = im->init(hD, hDsq, hNx, hinterp, hjxr);
    e->impl = std::move(im);
  } else {
    return slab::set_error(SLAB_ERR_ARG, "slab_engine_create: unknown precision %d", precision);
  }
  if (st != SLAB_OK) return st;
  *out = e.release();
  return SLAB_OK;
}

extern "C" int slab_engine_create(slab_engine** out, int p, int n0, int n1, int buf, int precision,
                                  const double* hD, const double* hDsq, const double* hNx, const double* hinterp,
                                  const int* hjxr, void* stream) {
  return engine_create(out, p, n0, n1, buf, precision, hD, hDsq, hNx, hinterp, hjxr, stream, false);
}

extern "C" int slab_engine_create_mixed(slab_engine** out, int p, int n0, int n1, int buf, int precision,
                                        const double* hD, const double* hDsq, const double* hNx,
                                        const double* hinterp, const int* hjxr, void* stream) {
  return engine_create(out, p, n0, n1, buf, precision, hD, hDsq, hNx, hinterp, hjxr, stream, true);
}

extern "C" int slab_engine_destroy(slab_engine* e) {
  delete e;
  return SLAB_OK;
}

extern "C" long long slab_launch_count(void) { return slab::launch_count(); }

extern "C" int slab_engine_timings(const slab_engine* e, double* ms, int n) {
  if (!e || !ms) return slab::set_error(SLAB_ERR_ARG, "slab_engine_timings: null argument");
  const int m = n < 6 ? n : 6;
  for (int i = 0; i < m; ++i) ms[i] = e->impl->timing(i);
  return m;
}

extern "C" int slab_engine_set_option(slab_engine* e, int key, int value) {
  if (!e) return slab::set_error(SLAB_ERR_ARG, "slab_engine_set_option: null engine");
  return e->impl->set_option(key, value);
}

extern "C" int slab_engine_get_option(const slab_engine* e, int key) {
  if (!e) return slab::set_error(SLAB_ERR_ARG, "slab_engine_get_option: null engine");
  return e->impl->get_option(key);
}

extern "C" long long slab_engine_nfaces(const slab_engine* e) { return e ? e->impl->ntot : -1; }
extern "C" long long slab_engine_nleaves(const slab_engine* e) { return e ? e->impl->nleaf : -1; }
extern "C" size_t slab_engine_factor_bytes(const slab_engine* e) { return e ? e->impl->factor_bytes() : 0; }
extern "C" size_t slab_engine_solve_bytes(const slab_engine* e) { return e ? e->impl->solve_bytes() : 0; }

extern "C" int slab_engine_factor(slab_engine* e, const double* c11, const double* c22, const double* c1,
                                  const double* c2, const double* c) {
  if (!e) return slab::set_error(SLAB_ERR_ARG, "slab_engine_factor: null engine");
  return e->impl->factor(slab::LeafCoeffs{c11, c22, c1, c2, c});
}

extern "C" int slab_engine_factor_mixed(slab_engine* e, const double* c11, const double* c22, const double* c12,
                                        const double* c1, const double* c2, const double* c) {
  if (!e) return slab::set_error(SLAB_ERR_ARG, "slab_engine_factor_mixed: null engine");
  return e->impl->factor(slab::LeafCoeffs{c11, c22, c1, c2, c, c12});
}

extern "C" int slab_engine_solve(slab_engine* e, int nrhs, const double* bnd, const double* fbody, double tol,
                                 int max_iter, double* ufaces, double* uleaf, int* iters, double* stats) {
  if (!e) return slab::set_error(SLAB_ERR_ARG, "slab_engine_solve: null engine");
  return e->impl->solve(nrhs, bnd, fbody, tol, max_iter, ufaces, uleaf, iters, stats);
}

// ---------------------------------------------------------------------------
// Several refined solves (independent engines, any sizes) as one CUDA graph.
struct slab_solve_graph {
  std::vector<slab_engine*> engines;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev = nullptr;
  std::vector<cudaEvent_t> eng_ev;
  std::vector<long long> epoch;  // engine buffer epochs at capture
  std::vector<char> counted;      // kernels of the last launch added to the count
};

extern "C" int slab_solve_graph_destroy(slab_solve_graph* g) {
  if (!g) return SLAB_OK;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  if (g->ev) cudaEventDestroy(g->ev);
  for (cudaEvent_t e : g->eng_ev)
    if (e) cudaEventDestroy(e);
  delete g;
  return SLAB_OK;
}

extern "C" int slab_solve_graph_create(slab_solve_graph** out, slab_engine* const* engines, int count, const int* nrhs,
                                       const double* const* bnd, const double* const* fbody, double* const* uleaf,
                                       double tol, int max_iter) {
  if (!out || !engines || count <= 0 || !nrhs || !bnd || !uleaf)
    return slab::set_error(SLAB_ERR_ARG, "slab_solve_graph_create: invalid arguments");
  *out = nullptr;
  for (int i = 0; i < count; ++i) {
    if (!engines[i]) return slab::set_error(SLAB_ERR_ARG, "slab_solve_graph_create: null engine %d", i);
    for (int j = 0; j < i; ++j)
      if (engines[j] == engines[i])
        return slab::set_error(SLAB_ERR_ARG, "slab_solve_graph_create: engine %d appears twice", i);
  }
  auto* g = new slab_solve_graph();
  g->engines.assign(engines, engines + count);
  int st = SLAB_OK;
  if (cudaGraphCreate(&g->graph, 0) != cudaSuccess || cudaEventCreateWithFlags(&g->ev, cudaEventDisableTiming) != cudaSuccess)
    st = slab::set_error(SLAB_ERR_CUDA, "slab_solve_graph_create: graph creation failed");
  for (int i = 0; i < count && st == SLAB_OK; ++i)
    st = engines[i]->impl->capture_solve(g->graph, nrhs[i], bnd[i], fbody ? fbody[i] : nullptr, uleaf[i], tol,
                                         max_iter);
  if (st == SLAB_OK) {
    const cudaError_t e = cudaGraphInstantiate(&g->exec, g->graph, 0);
    if (e != cudaSuccess) {
      g->exec = nullptr;
      st = slab::set_error(SLAB_ERR_CUDA, "slab_solve_graph_create: instantiate: %s", cudaGetErrorString(e));
    }
  }
  g->eng_ev.assign(count, nullptr);
  g->counted.assign(count, 1);
  for (int i = 0; i < count; ++i) g->epoch.push_back(engines[i]->impl->epoch());
  for (int i = 0; i < count && st == SLAB_OK; ++i)
    if (cudaEventCreateWithFlags(&g->eng_ev[i], cudaEventDisableTiming) != cudaSuccess)
      st = slab::set_error(SLAB_ERR_CUDA, "slab_solve_graph_create: event creation failed");
  if (st != SLAB_OK) {
    slab_solve_graph_destroy(g);
    return st;
  }
  *out = g;
  return SLAB_OK;
}

extern "C" int slab_solve_graph_launch(slab_solve_graph* g, void* stream) {
  if (!g || !g->exec) return slab::set_error(SLAB_ERR_ARG, "slab_solve_graph_launch: no graph");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  for (size_t i = 0; i < g->engines.size(); ++i)
    if (g->engines[i]->impl->epoch() != g->epoch[i])
      return slab::set_error(SLAB_ERR_STATE,
                             "slab_solve_graph_launch: engine %zu reallocated its buffers after the graph was made "
                             "(a solve with more right-hand sides or another set of coefficients); create a new graph",
                             i);
  // after the engines' earlier work (their factorizations); before their later work
  for (size_t i = 0; i < g->engines.size(); ++i) {
    SLAB_CUDA_TRY(cudaEventRecord(g->eng_ev[i], g->engines[i]->impl->stream()));
    SLAB_CUDA_TRY(cudaStreamWaitEvent(s, g->eng_ev[i], 0));
  }
  SLAB_CUDA_TRY(cudaGraphLaunch(g->exec, s));
  SLAB_CUDA_TRY(cudaEventRecord(g->ev, s));
  g->counted.assign(g->engines.size(), 0);
  for (slab_engine* e : g->engines) SLAB_CUDA_TRY(cudaStreamWaitEvent(e->impl->stream(), g->ev, 0));
  return SLAB_OK;
}

extern "C" int slab_solve_graph_status(slab_solve_graph* g, int i, int* iters, double* stats) {
  if (!g || i < 0 || i >= (int)g->engines.size()) return slab::set_error(SLAB_ERR_ARG, "slab_solve_graph_status: index");
  SLAB_CUDA_TRY(cudaEventSynchronize(g->ev));
  const bool count = !g->counted[i];
  g->counted[i] = 1;
  return g->engines[i]->impl->graph_status(iters, stats, count);
}

extern "C" int slab_engine_adjoint(slab_engine* e, int nrhs, const double* gleaf, const double* gfaces, double tol,
                                   int max_iter, double* lam_leaf, double* lam_faces, double* gbnd, int* iters,
                                   double* stats) {
  if (!e) return slab::set_error(SLAB_ERR_ARG, "slab_engine_adjoint: null engine");
  return e->impl->adjoint(nrhs, gleaf, gfaces, tol, max_iter, lam_leaf, lam_faces, gbnd, iters, stats);
}

extern "C" int slab_engine_coeff_grad(slab_engine* e, int nrhs, const double* ufaces, const double* uleaf,
                                      const double* lam_leaf, double* g11, double* g22, double* g1, double* g2,
                                      double* g) {
  if (!e) return slab::set_error(SLAB_ERR_ARG, "slab_engine_coeff_grad: null engine");
  return e->impl->coeff_grad(nrhs, ufaces, uleaf, lam_leaf, g11, g22, nullptr, g1, g2, g);
}

extern "C" int slab_engine_coeff_grad_mixed(slab_engine* e, int nrhs, const double* ufaces, const double* uleaf,
                                            const double* lam_leaf, double* g11, double* g22, double* g12,
                                            double* g1, double* g2, double* g) {
  if (!e) return slab::set_error(SLAB_ERR_ARG, "slab_engine_coeff_grad_mixed: null engine");
  return e->impl->coeff_grad(nrhs, ufaces, uleaf, lam_leaf, g11, g22, g12, g1, g2, g);
}

extern "C" int slab_engine_apply(slab_engine* e, int nrhs, const double* rint, const double* rfaces, double* dint,
                                 double* dfaces) {
  if (!e) return slab::set_error(SLAB_ERR_ARG, "slab_engine_apply: null engine");
  return e->impl->apply_once(nrhs, rint, rfaces, dint, dfaces);
}

extern "C" int slab_engine_residual(slab_engine* e, int nrhs, const double* ufaces, const double* uint,
                                    const double* fbody, double* rint, double* rfaces) {
  if (!e) return slab::set_error(SLAB_ERR_ARG, "slab_engine_residual: null engine");
  return e->impl->residual(nrhs, ufaces, uint, fbody, rint, rfaces);
}
