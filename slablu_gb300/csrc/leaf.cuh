// Leaf-level kernels of the HPS discretisation (unit-square leaves, c12 = None).
#pragma once

#include "dense.cuh"

namespace slab {

// Canonical leaf node of interior row r (Jc order) and of face-node column s
// (Jx = [Jl, Jr, Jd, Ju]); node = i1*p + i2 (src_disc/hps_subdomain_disc.py:105-134).
__host__ __device__ inline void interior_node(int r, int q, int& i1, int& i2) {
  i1 = r / q + 1;
  i2 = r % q + 1;
}
__host__ __device__ inline void face_node(int s, int p, int q, int& j1, int& j2) {
  const int f = s / q, t = s % q + 1;
  switch (f) {
    case 0: j1 = 0; j2 = t; break;
    case 1: j1 = p - 1; j2 = t; break;
    case 2: j1 = t; j2 = 0; break;
    default: j1 = t; j2 = p - 1; break;
  }
}

struct LeafCoeffs {
  const double* c11;
  const double* c22;
  const double* c1;
  const double* c2;
  const double* c;
  const double* c12 = nullptr;  // mixed derivative (read by the kMixed kernels only)
};

template <typename T>
struct LeafFactorArgs {
  int p, q, n, nx;
  LeafCoeffs co;            // nleaf*p*p each (offset to the first leaf of the launch) or null
  const double* D;          // p*p row-major
  const double* Dsq;        // p*p row-major
  const T* Nxc;             // nx x n   column-major
  const T* Nxx;             // nx x nx  column-major
  T* G;                     // per leaf n x (n+nx) column-major (ld n): LU | S
  long long strideG;
  int* piv;                 // per leaf n
  T* dtn;                   // per leaf nx x nx column-major
  int* info;                // per leaf
  int decouple;             // replace Dirichlet-face rows/cols by identity
  int n0, n1, leaf_begin;   // grid geometry (for decouple)
  // mixed derivative (co.c12): the extra columns are the nxa = 4(p-1) nodes
  // jxr (Jxreorder, corners included) and S = -A_cc^{-1} A_c,jxr interp with
  // interp (nxa x nx, row-major); nxa = 0 means the nx face nodes
  int nxa;
  const T* interp;
  const int* jxr;
  // [A_cc | A_cx] already written into G by leaf_assemble_kernel (no mixed
  // derivative): the factor kernel starts at the LU
  int preassembled = 0;
};

// Entry (row node k=(i1,i2), column node (j1,j2)) of
//   Aloc = -c11 D11 - c22 D22 - 2 c12 D12 + c1 D1 + c2 D2 + diag(c)
// accumulated in the reference's term order (src_disc/hps_parallel_leaf_ops.py:17-27);
// D12 = kron(D, D), so its entry is the single product D[i1,j1] D[i2,j2].  The
// c12 term exists only in the kMixed instantiation.
template <bool kMixed = false>
__device__ __forceinline__ double aloc_entry(const LeafCoeffs& co, int lofs, int p, int i1, int i2, int j1,
                                             int j2, const double* D, const double* Dsq) {
  const int k = lofs + i1 * p + i2;
  double v = 0.0;
  if (i2 == j2 && co.c11) v += (-co.c11[k]) * Dsq[i1 * p + j1];
  if (i1 == j1 && co.c22) v += (-co.c22[k]) * Dsq[i2 * p + j2];
  if (kMixed && co.c12) v += (-2.0 * co.c12[k]) * (D[i1 * p + j1] * D[i2 * p + j2]);
  if (i2 == j2 && co.c1) v += co.c1[k] * (-D[i1 * p + j1]);
  if (i1 == j1 && co.c2) v += co.c2[k] * (-D[i2 * p + j2]);
  if (i1 == j1 && i2 == j2 && co.c) v += co.c[k];
  return v;
}

// Shared-memory bytes of the assembly stage of leaf_factor_kernel: D, Dsq and
// the leaf's six coefficient fields (FP64, p*p each) and the (i1, i2) node
// indices of every interior row.  They occupy the start of the dynamic region,
// which the LU reuses once assembly is done.
inline size_t leaf_assembly_smem_bytes(int p) {
  const int n = (p - 2) * (p - 2);
  return 8 * (size_t)p * p * sizeof(double) + 2 * (size_t)n;
}

// Dynamic shared memory of leaf_factor_kernel<T> for order p.
inline size_t leaf_factor_smem_bytes(int p, size_t elem) {
  const int n = (p - 2) * (p - 2);
  const size_t b = (size_t)getrf_smem_elems(n) * elem;
  const size_t asm_b = leaf_assembly_smem_bytes(p);
  return b > asm_b ? b : asm_b;
}

// One CTA per leaf: assemble [A_cc | A_cx], pivoted LU, S = -A_cc^{-1} A_cx,
// DtN = Nx[:,Jc] S + Nx[:,Jx] (src_disc/hps_parallel_leaf_ops.py:40-58).
// kMixed: the operator has a mixed derivative c12 (:59-65): the extra columns
// are the 4(p-1) nodes Jxreorder (corners included), and after the back
// substitution X = A_cc^{-1} A_c,Jxreorder is replaced by X Interp_mat.
// Assembly of [A_cc | A_cx] (no mixed derivative) for every leaf into G, in the
// layout and term order of leaf_factor_kernel's own assembly: one CTA per leaf
// with the leaf's coefficients and D, Dsq staged in shared memory, one warp per
// column.  Separate from the factorization, the FP64 evaluation of the entries
// runs at full occupancy instead of inside the latency-bound factor kernel.
template <typename T>
__global__ void __launch_bounds__(kNT) leaf_assemble_kernel(LeafFactorArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x, leaf = blockIdx.x;
  const int p = a.p, q = a.q, n = a.n, nx = a.nx, pp = p * p;
  double* Dsh = reinterpret_cast<double*>(smem_raw);
  double* Dsqsh = Dsh + pp;
  double* csh = Dsqsh + pp;
  const int lofs = leaf * pp;
  LeafCoeffs cs{};
  {
    const double* src[5] = {a.co.c11, a.co.c22, a.co.c1, a.co.c2, a.co.c};
    const double** dst[5] = {&cs.c11, &cs.c22, &cs.c1, &cs.c2, &cs.c};
#pragma unroll
    for (int f = 0; f < 5; ++f) {
      if (!src[f]) continue;
      double* d = csh + f * pp;
      for (int i = tid; i < pp; i += blockDim.x) d[i] = src[f][lofs + i];
      *dst[f] = d;
    }
  }
  unsigned char* ri1 = reinterpret_cast<unsigned char*>(csh + 5 * pp);
  unsigned char* ri2 = ri1 + n;
  for (int i = tid; i < pp; i += blockDim.x) {
    Dsh[i] = a.D[i];
    Dsqsh[i] = a.Dsq[i];
  }
  for (int r = tid; r < n; r += blockDim.x) {
    int i1, i2;
    interior_node(r, q, i1, i2);
    ri1[r] = (unsigned char)i1;
    ri2[r] = (unsigned char)i2;
  }
  __syncthreads();
  T* G = a.G + a.strideG * leaf;
  const int nc = n + nx;
  const int lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  for (int col = warp; col < nc; col += nwarps) {
    int j1, j2;
    if (col < n)
      interior_node(col, q, j1, j2);
    else
      face_node(col - n, p, q, j1, j2);
    T* gc = G + (size_t)col * n;
    for (int r = lane; r < n; r += 32) {
      const int i1 = ri1[r], i2 = ri2[r];
      T v = T(0);
      if (i1 == j1 || i2 == j2) v = (T)aloc_entry<false>(cs, 0, p, i1, i2, j1, j2, Dsh, Dsqsh);
      gc[r] = v;
    }
  }
}

template <typename T, bool kMixed = false>
__global__ void __launch_bounds__(kNT) leaf_factor_kernel(LeafFactorArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x;
  const int leaf = blockIdx.x;
  const int p = a.p, q = a.q, n = a.n, nx = a.nx;
  T* smem = reinterpret_cast<T*>(smem_raw);
  const int pp = p * p;
  T* G = a.G + a.strideG * leaf;
  const int nxa = kMixed ? a.nxa : nx;  // extra columns: face nodes, or Jxreorder with c12
  const int nc = n + nxa;
  if (kMixed || !a.preassembled) {
  double* Dsh = reinterpret_cast<double*>(smem_raw);
  double* Dsqsh = Dsh + pp;
  // the leaf's coefficients in shared memory: the assembly reads each of them
  // many times, and from global memory every read would be a dependent round trip
  double* csh = Dsqsh + pp;
  const int lofs = leaf * pp;
  LeafCoeffs cs{};
  constexpr int kNF = kMixed ? 6 : 5;  // coefficient fields staged
  {
    const double* src[6] = {a.co.c11, a.co.c22, a.co.c1, a.co.c2, a.co.c, a.co.c12};
    const double** dst[6] = {&cs.c11, &cs.c22, &cs.c1, &cs.c2, &cs.c, &cs.c12};
#pragma unroll
    for (int f = 0; f < kNF; ++f) {
      if (!src[f]) continue;
      double* d = csh + f * pp;
      for (int i = tid; i < pp; i += blockDim.x) cp_async_elem(&d[i], &src[f][lofs + i]);
      *dst[f] = d;
    }
  }
  unsigned char* ri1 = reinterpret_cast<unsigned char*>(csh + kNF * pp);  // x index of interior row r
  unsigned char* ri2 = ri1 + n;                                         // y index
  for (int i = tid; i < pp; i += blockDim.x) {
    Dsh[i] = a.D[i];
    Dsqsh[i] = a.Dsq[i];
  }
  for (int r = tid; r < n; r += blockDim.x) {
    int i1, i2;
    interior_node(r, q, i1, i2);
    ri1[r] = (unsigned char)i1;
    ri2[r] = (unsigned char)i2;
  }
  cp_async_wait_all();
  __syncthreads();
  // one warp per column: without c12, Aloc[Jc, col] is nonzero only on the rows
  // that share the column node's x or y line
  {
    const int lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    for (int col = warp; col < nc; col += nwarps) {
      int j1, j2;
      if (col < n) {
        interior_node(col, q, j1, j2);
      } else if (kMixed) {
        const int t = a.jxr[col - n];
        j1 = t / p;
        j2 = t % p;
      } else {
        face_node(col - n, p, q, j1, j2);
      }
      T* gc = G + (size_t)col * n;
      for (int r = lane; r < n; r += 32) {
        const int i1 = ri1[r], i2 = ri2[r];
        // zeros are stored as T directly: an FP64 -> FP32 conversion runs at
        // the FP64 rate, which is 1/64 of FP32 on this GPU
        T v = T(0);
        if (kMixed || i1 == j1 || i2 == j2) v = (T)aloc_entry<kMixed>(cs, 0, p, i1, i2, j1, j2, Dsh, Dsqsh);
        gc[r] = v;
      }
    }
  }
  }  // assembly
  __syncthreads();
  cta_getrf_aug<T>(G, n, n, nc, a.piv + (size_t)leaf * n, smem, a.info ? a.info + leaf : nullptr);
  for (int c0 = 0; c0 < nxa; c0 += kCT) cta_backsub<T>(G, n, n, n + c0, min(kCT, nxa - c0), smem);
  if constexpr (kMixed) {
    // X Interp_mat in place of the first nx extra columns, 32 rows at a time
    // (each chunk's rows are read completely before they are overwritten;
    // cta_backsub ends with a block barrier, so the staging area is free)
    constexpr int kR = 32;
    T* Is = smem;                    // nxa x nx, row-major
    T* Xc = Is + (size_t)nxa * nx;   // kR x nxa
    for (int idx = tid; idx < nxa * nx; idx += blockDim.x) Is[idx] = a.interp[idx];
    for (int r0 = 0; r0 < n; r0 += kR) {
      const int rr = min(kR, n - r0);
      __syncthreads();
      for (int idx = tid; idx < rr * nxa; idx += blockDim.x) {
        const int r = idx % rr, t = idx / rr;
        Xc[r + t * kR] = G[(size_t)(n + t) * n + r0 + r];
      }
      __syncthreads();
      for (int idx = tid; idx < rr * nx; idx += blockDim.x) {
        const int r = idx % rr, c = idx / rr;
        T v = T(0);
        for (int t = 0; t < nxa; ++t) v += Xc[r + t * kR] * Is[(size_t)t * nx + c];
        G[(size_t)(n + c) * n + r0 + r] = v;
      }
    }
  }
  // DtN = Nxx - Nxc X  (X = A_cc^{-1} A_cx, S = -X)
  T* dtn = a.dtn + (size_t)leaf * nx * nx;
  for (int idx = tid; idx < nx * nx; idx += blockDim.x) dtn[idx] = a.Nxx[idx];
  T* Psm = smem;
  T* Bt = smem + round_up(n, 4) * kNB + kPad;
  const int ldq = round_up(nx, 4);
  const T* X = G + (size_t)n * n;
  for (int k0 = 0; k0 < n; k0 += kNB) {
    const int kb = min(kNB, n - k0);
    __syncthreads();
    for (int c = 0; c < kb; ++c)
      for (int r = tid; r < nx; r += blockDim.x) cp_async_elem(&Psm[r + c * ldq], &a.Nxc[r + (size_t)(k0 + c) * nx]);
    for (int idx = tid; idx < kb * nx; idx += blockDim.x) {
      const int kk = idx % kb, c = idx / kb;
      cp_async_elem(&Bt[c + kk * kCTLD], &X[(size_t)c * n + k0 + kk]);
    }
    cp_async_wait_all();
    __syncthreads();
    cta_gemm_sub(dtn, nx, nx, nx, Psm, ldq, Bt, kCTLD, kb);
  }
  __syncthreads();
  for (int idx = tid; idx < n * nx; idx += blockDim.x) G[(size_t)n * n + idx] = -G[(size_t)n * n + idx];
  if (a.decouple) {
    const int gl = a.leaf_begin + leaf;
    const int I = gl / a.n1, J = gl % a.n1;
    const bool dir[4] = {I == 0, I == a.n0 - 1, J == 0, J == a.n1 - 1};
    if (dir[0] || dir[1] || dir[2] || dir[3]) {
      for (int idx = tid; idx < nx * nx; idx += blockDim.x) {
        const int r = idx % nx, c = idx / nx;
        if (dir[r / q] || dir[c / q]) dtn[idx] = r == c ? T(1) : T(0);
      }
    }
  }
}

// ctas_per_sm > 0 sizes the dynamic shared memory so that at most that many
// leaves are resident per SM (fewer resident leaves keep more of each leaf's
// trailing matrix in L2); 0 uses the minimum size.
template <typename T>
int leaf_factor(cudaStream_t s, const LeafFactorArgs<T>& a, int nleaf, int ctas_per_sm = 0);

// Dynamic shared-memory bytes (at least `need`) that allow at most ctas_per_sm
// resident blocks of `kernel` per SM; `need` itself when ctas_per_sm <= 0.
size_t leaf_smem_for_occupancy(const void* kernel, size_t need, int ctas_per_sm);

// Nx (nx x p^2 row-major, FP64) -> Nxc (nx x n) and Nxx (nx x nx), column-major, in T.
template <typename T>
__global__ void split_nx_kernel(const double* Nx, int p, int q, T* Nxc, T* Nxx) {
  const int nx = 4 * q, n = q * q;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < nx * (n + nx); idx += gridDim.x * blockDim.x) {
    const int t = idx % nx, col = idx / nx;
    int j1, j2;
    if (col < n) {
      interior_node(col, q, j1, j2);
      Nxc[t + (size_t)col * nx] = (T)Nx[(size_t)t * p * p + j1 * p + j2];
    } else {
      face_node(col - n, p, q, j1, j2);
      Nxx[t + (size_t)(col - n) * nx] = (T)Nx[(size_t)t * p * p + j1 * p + j2];
    }
  }
}

// ---------------------------------------------------------------------------
// FP64 residual of the full collocation system, one CTA per leaf.
struct ResidualArgs {
  int p, q, n, nx, nleaf, nrhs;
  long long ntot;
  LeafCoeffs co;
  const double* D;
  const double* Dsq;
  const int* leafglob;          // nleaf x nx global face-node index of each leaf face node
  const unsigned char* dirmask; // ntot: 1 on Dirichlet face nodes
  const double* ux;             // ntot x nrhs
  const double* uc;             // leaf-major: leaf*n*nrhs + c*n + r
  const double* fbody;          // (nleaf*p*p) x nrhs column-major, or null
  double* rc;                   // leaf-major like uc
  double* rx;                   // ntot x nrhs, accumulated with atomicAdd (caller zeroes)
  int all_faces;                // residual_t_kernel: also accumulate into Dirichlet face columns
  // residual_mixed_kernel only: Interp_mat (nxa x nx, row-major) and the Jxreorder nodes
  const double* interp;
  const int* jxr;
  int nxa;
};

__global__ void residual_kernel(ResidualArgs a);

// The residual with a mixed derivative c12 (shared memory (4 p^2 + nx) doubles):
// the PDE rows see the interpolated boundary u[Jxreorder] = Interp_mat u_faces
// (corners included) and carry -2 c12 (D U D^T); the flux rows see the face
// values themselves -- the split of the reference's c12 branch, whose leaf
// solve interpolates the boundary and whose DtN map is Nx[:,Jc] S + Nx[:,Jx]
// (src_disc/hps_parallel_leaf_ops.py:59-65, 84-92).
__global__ void residual_mixed_kernel(ResidualArgs a);

// FP64 residual of the transposed system, one CTA per leaf:
//   rc = g_int - (A^T lam) at interior columns (leaf-major, like uc),
//   rx -= (A^T lam) at face columns (caller initialises rx to g_faces),
// with lam = (uc, ux) holding the multipliers of the interior PDE rows and of
// the face flux rows (ux is read as zero on Dirichlet faces, which have no
// row).  fbody holds g_int in the leaf-major interior layout.  Dirichlet face
// columns are skipped unless all_faces is set; with it, rx there becomes the
// sensitivity of the loss to the Dirichlet data.
__global__ void residual_t_kernel(ResidualArgs a);

// The same with a mixed derivative c12 (interp, jxr, nxa as for
// residual_mixed_kernel; shared memory (9 p^2 + nx) doubles): the PDE rows'
// part of A^T lam is formed at every leaf node, corners included, and reaches
// the face columns through Interp_mat^T; the flux rows' part (Nx^T lam_x) is
// added at the interior and face nodes.
__global__ void residual_t_mixed_kernel(ResidualArgs a);

// Adjoint of the solution assembly (sol_tot from interior and face values):
// dsol (nleaf*p*p x nrhs, column-major) -> g_int = dsol at interior nodes
// (leaf-major) and g_faces += Interp^T dsol at the leaf boundary nodes
// (atomically, every face including Dirichlet ones).
struct AssembleTArgs {
  int p, q, n, nx, nleaf, nrhs;
  long long ntot;
  const int* leafglob;
  const double* interp;
  const int* jxreorder;
  const double* dsol;
  double* gint;
  double* gfaces;
};
__global__ void assemble_t_kernel(AssembleTArgs a);

// Coefficient gradients of a loss L(u) where A(c) u = f, from the multipliers
// lam of the interior PDE rows: with (A u)_k = -c11 t11 - c22 t22 - c1 t1 -
// c2 t2 + c u_k (t11 = (D11 u)_k, t1 = (-D1 u)_k, ...),
//   dL/dc_k = -lam_k u_k, dL/dc11_k = lam_k t11, dL/dc22_k = lam_k t22,
//   dL/dc1_k = lam_k t1,  dL/dc2_k = lam_k t2
// at interior nodes k (zero at leaf boundary nodes), summed over the
// right-hand sides.  u: interior values from uleaf, face values from ufaces.
struct GradArgs {
  int p, q, n, nx, nleaf, nrhs;
  long long ntot;
  const double* D;
  const double* Dsq;
  const int* leafglob;
  const double* uleaf;   // nleaf*p*p x nrhs column-major
  const double* ufaces;  // ntot x nrhs
  const double* lam;     // nleaf*p*p x nrhs column-major (interior nodes read)
  double* g11;
  double* g22;
  double* g1;
  double* g2;
  double* g0;            // each nleaf*p*p or null
  // coeff_grad_mixed_kernel only: dL/dc12 (or null), Interp_mat (nxa x nx,
  // row-major) and the Jxreorder nodes
  double* g12;
  const double* interp;
  const int* jxr;
  int nxa;
};
__global__ void coeff_grad_kernel(GradArgs a);

// The same for an operator with a mixed derivative (shared memory (4 p^2 + nx)
// doubles): every term is evaluated on the node values the PDE rows see, the
// interior values and Interp_mat u_faces on the leaf boundary (corners
// included); with (A u)_k carrying -2 c12_k (D12 u)_k, dL/dc12_k =
// 2 lam_k (D12 u)_k.
__global__ void coeff_grad_mixed_kernel(GradArgs a);

// sol_tot assembly: out[(leaf*p*p + k) + c*nleaf*p*p] for every leaf node.
struct AssembleArgs {
  int p, q, n, nx, nleaf, nrhs;
  long long ntot;
  const int* leafglob;
  const double* interp;   // 4(p-1) x nx row-major
  const int* jxreorder;   // 4(p-1)
  const double* ux;       // ntot x nrhs
  const double* uc;       // leaf-major
  double* out;
  const int* ispan;       // per row of interp [first, last + 1) nonzero column, or null (all nx)
};

// Right-hand sides assembled together by one CTA (shared memory nx x this doubles).
constexpr int kAssembleRhs = 8;
__global__ void assemble_solution_kernel(AssembleArgs a);

}  // namespace slab
