/*
 * slablu_gb300 -- C ABI of the GB300-native SlabLU factor-and-solve path.
 *
 * Conventions shared by every entry point:
 *   - pointers named d_* are device pointers (CUDA global memory of the current
 *     device); h_* are host pointers.  Nothing in this header takes a torch type.
 *   - dense matrices crossing the ABI are row-major (C order), as the reference's
 *     torch/NumPy tensors are.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *   - return value: SLAB_OK (0); > 0 is a pivot breakdown in the LAPACK `info`
 *     sense (1-based column of the first exactly-zero pivot); < 0 is an error
 *     code below.  slab_last_error() describes the most recent failure of the
 *     calling thread.
 *   - leaf discretisation conventions are the reference's
 *     (src_disc/hps_subdomain_disc.py:105-152): p x p tensor Chebyshev nodes,
 *     node k = i1*p + i2 with i1 the x index; interior nodes Jc in ascending
 *     order; face nodes Jx = [Jl, Jr, Jd, Ju]; D is the 1-D derivative matrix
 *     (scaled by 1/a) with D1 = -kron(D, I), D2 = -kron(I, D), Dsq = D @ D.
 *   - reduced face unknowns are numbered as the reference numbers them
 *     (src_disc/hps_multidomain_disc.py:63-81): face f, node k -> f*(p-2) + k.
 */
#ifndef SLABLU_GB300_H
#define SLABLU_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SLAB_OK 0
#define SLAB_ERR_ARG (-1)
#define SLAB_ERR_CUDA (-2)
#define SLAB_ERR_ALLOC (-3)
#define SLAB_ERR_STATE (-4)
#define SLAB_ERR_NOCONV (-5)

/* Arithmetic of the factorization. */
#define SLAB_PREC_FP64 0  /* everything in FP64                                         */
#define SLAB_PREC_MIXED 1 /* FP32 leaf + slab factors, FP64 interface LU, FP64 residual */
#define SLAB_PREC_FP32 2  /* FP32 factors everywhere, FP64 residual                     */

/* Library version as an integer (major*10000 + minor*100 + patch). */
int slab_version(void);

/* Human-readable description of the last error on this thread. */
const char* slab_last_error(void);

/*
 * Batched leaf Dirichlet-to-Neumann maps.
 * Replaces form_DtNs(mode='build') and get_DtNs_helper
 * (src_disc/hps_parallel_leaf_ops.py:40-72, :113-140) for the c12 = None case:
 *   Aloc = -c11 D11 - c22 D22 + c1 D1 + c2 D2 + diag(c)      (:10-37)
 *   S    = -Aloc[Jc,Jc]^{-1} Aloc[Jc,Jx]
 *   DtN  = Nx[:,Jc] S + Nx[:,Jx]
 * d_c11 .. d_c: coefficient values at the p*p nodes of each leaf, nleaf*p*p
 *   doubles each, or NULL for an absent term (c11/c22 NULL mean zero).
 * d_D, d_Dsq: p*p doubles.  d_Nx: 4(p-2) x p*p doubles (HPS_Disc.Nx).
 * precision: SLAB_PREC_FP64 or SLAB_PREC_FP32 (factor arithmetic).
 * d_work: scratch of slab_leaf_dtn_work_bytes() bytes (holds the leaf LU factors).
 * d_dtn: nleaf x 4(p-2) x 4(p-2) doubles (row-major per leaf).
 * d_S: optional (NULL) nleaf x (p-2)^2 x 4(p-2) doubles receiving S.
 * d_info: nleaf ints, per-leaf LAPACK-style info (0 = success).
 */
size_t slab_leaf_dtn_work_bytes(int nleaf, int p, int precision);
int slab_leaf_dtn(int nleaf, int p, const double* d_c11, const double* d_c22, const double* d_c1,
                  const double* d_c2, const double* d_c, const double* d_D, const double* d_Dsq,
                  const double* d_Nx, int precision, void* d_work, size_t work_bytes, double* d_dtn,
                  double* d_S, int* d_info, void* stream);

/*
 * Batched leaf DtN maps with a mixed-derivative term (c12, for the parameter maps of
 * curved domains).  Replaces the c12 branch of form_DtNs(mode='build')
 * (src_disc/hps_parallel_leaf_ops.py:59-65):
 *   Aloc = -c11 D11 - c22 D22 - 2 c12 D12 + c1 D1 + c2 D2 + diag(c)   (D12 = kron(D, D))
 *   S    = -Aloc[Jc,Jc]^{-1} Aloc[Jc,Jxreorder] Interp_mat
 *   DtN  = Nx[:,Jc] S + Nx[:,Jx]
 * d_interp: 4(p-1) x 4(p-2) doubles, row-major (HPS_Disc.Interp_mat);
 * d_jxreorder: 4(p-1) ints (JJ.Jxreorder).  Other arguments as slab_leaf_dtn,
 * with a work area of slab_leaf_dtn_mixed_work_bytes() bytes; d_c12 NULL gives
 * the slab_leaf_dtn result.
 */
size_t slab_leaf_dtn_mixed_work_bytes(int nleaf, int p, int precision);
int slab_leaf_dtn_mixed(int nleaf, int p, const double* d_c11, const double* d_c22, const double* d_c12,
                        const double* d_c1, const double* d_c2, const double* d_c, const double* d_D,
                        const double* d_Dsq, const double* d_Nx, const double* d_interp, const int* d_jxreorder,
                        int precision, void* d_work, size_t work_bytes, double* d_dtn, double* d_S, int* d_info,
                        void* stream);

/*
 * Allocation-free batched leaf DtN maps.  No counterpart in the reference: it
 * exists for callers that cannot allocate device memory when they need DtN
 * maps (a host application whose own pool allocator owns all device memory and
 * forbids library allocations, or a program with a device-memory budget fixed
 * at start-up).  Same arguments and
 * results as slab_leaf_dtn without the work buffer and without S; the leaf
 * factors live in a fixed scratch array compiled into the library
 * (slab_leaf_dtn_noalloc_max_bytes() bytes, held on every device that loads
 * the library).  Calls whose work would exceed it fail with SLAB_ERR_ARG.
 * The first call on each device looks up the scratch address
 * (cudaGetSymbolAddress) and should come before any stream capture.  All
 * calls share the scratch: calls that overlap on the GPU race.  Allocates
 * nothing (no cudaMalloc / cudaFree).
 */
size_t slab_leaf_dtn_noalloc_max_bytes(void);
int slab_leaf_dtn_noalloc(int nleaf, int p, const double* d_c11, const double* d_c22, const double* d_c1,
                          const double* d_c2, const double* d_c, const double* d_D, const double* d_Dsq,
                          const double* d_Nx, int precision, double* d_dtn, int* d_info, void* stream);

/*
 * Factor-and-solve engine for the unit-square HPS SlabLU path.
 * Replaces Domain_Solver.build (src_solver/slablu_solver.py:440-487: leaf DtN
 * assembly, build_slabLU :297-358, build_Tred_solver :668-687) and
 * Domain_Solver.solve (:543-666 with leaf recovery,
 * src_disc/hps_multidomain_disc.py:227-243) for solver_type='slabLU',
 * non-periodic, c12 = None (c12: slab_engine_create_mixed).
 *
 * Geometry: n0 x n1 leaves (leaf index i*n1 + j, i = x index), polynomial
 * order p, slab width buf leaves (n0 % buf == 0).  Host arrays:
 *   h_D, h_Dsq  p*p doubles;  h_Nx 4(p-2) x p*p doubles;
 *   h_interp    4(p-1) x 4(p-2) doubles (HPS_Disc.Interp_mat);
 *   h_jxreorder 4(p-1) ints (JJ.Jxreorder).
 * The engine owns its device memory; it is not re-entrant; all work is
 * ordered on `stream`.
 */
typedef struct slab_engine slab_engine;

int slab_engine_create(slab_engine** out, int p, int n0, int n1, int buf, int precision, const double* h_D,
                       const double* h_Dsq, const double* h_Nx, const double* h_interp,
                       const int* h_jxreorder, void* stream);
int slab_engine_destroy(slab_engine* e);

/*
 * Engine for an operator with a mixed derivative (c12, the parameter maps of
 * curved domains): the c12 branch of form_DtNs (src_disc/hps_parallel_leaf_ops.py
 * :59-65, 84-92) -- leaves couple to their corners through Interp_mat.  Same
 * arguments as slab_engine_create; factor it with slab_engine_factor_mixed.
 * Solves, the residual and the adjoint work as for slab_engine_create; the
 * coefficient gradients, dL/dc12 included, come from
 * slab_engine_coeff_grad_mixed.
 */
int slab_engine_create_mixed(slab_engine** out, int p, int n0, int n1, int buf, int precision, const double* h_D,
                             const double* h_Dsq, const double* h_Nx, const double* h_interp,
                             const int* h_jxreorder, void* stream);

/* Number of reduced face unknowns (p-2)(n0(2 n1 + 1) + n1) and of leaves. */
long long slab_engine_nfaces(const slab_engine* e);
long long slab_engine_nleaves(const slab_engine* e);

/* Factor the operator with coefficients at every leaf node (nleaf*p*p
 * doubles each, NULL = absent).  Returns >0 on pivot breakdown. */
int slab_engine_factor(slab_engine* e, const double* d_c11, const double* d_c22, const double* d_c1,
                       const double* d_c2, const double* d_c);
/* The same with the mixed-derivative coefficient d_c12 (required), for an
 * engine from slab_engine_create_mixed:
 *   -c11 u_xx - c22 u_yy - 2 c12 u_xy + c1 u_x + c2 u_y + c u. */
int slab_engine_factor_mixed(slab_engine* e, const double* d_c11, const double* d_c22, const double* d_c12,
                             const double* d_c1, const double* d_c2, const double* d_c);

/*
 * Solve for nrhs right-hand sides with FP64 iterative refinement.
 * d_bnd:   nfaces x nrhs (column-major) face values; only the Dirichlet
 *          (domain-boundary) faces are read.
 * d_fbody: nleaf*p*p x nrhs body load at leaf nodes (column-major) or NULL.
 * tol:     stop when ||correction|| <= tol * ||solution|| (FP64 norms).
 * Outputs: d_ufaces nfaces x nrhs (column-major, may be NULL),
 *          d_uleaf  nleaf*p*p x nrhs solution at every leaf node (column-major,
 *                   corners and faces through Interp_mat as the reference does),
 *          h_iters  refinement steps taken,
 *          h_stats  5 doubles: [last relative correction, final residual norm,
 *                   initial residual norm, interior (leaf-local) residual norm,
 *                   relative residual].
 * Returns SLAB_ERR_NOCONV if max_iter steps did not reach tol (outputs hold
 * the last iterate).
 */
int slab_engine_solve(slab_engine* e, int nrhs, const double* d_bnd, const double* d_fbody, double tol,
                      int max_iter, double* d_ufaces, double* d_uleaf, int* h_iters, double* h_stats);

/*
 * The refined solves of several factored engines (any geometries, one engine
 * at most once) as one CUDA graph: per engine the set-up, a conditional WHILE
 * node whose body is one refinement step (FP64 residual, one application of
 * the factors, update; a one-thread kernel decides on the device whether
 * another step runs) and the final residual and assembly into d_uleaf[i].  A
 * launch needs no host round trip between steps and runs the engines'
 * solves side by side.  Same results as slab_engine_solve (the graph takes
 * one extra step when the first residual is exactly zero).
 *   count       : number of engines
 *   nrhs[i]     : right-hand sides of engine i
 *   d_bnd[i], d_fbody[i] (d_fbody may be NULL, as may its entries),
 *   d_uleaf[i]  : device buffers of the caller, laid out as for
 *                 slab_engine_solve, read and written at every launch
 * The graph reads each engine's current factors, so a re-factorization of the
 * same coefficient set is picked up by the next launch.  A launch fails with
 * SLAB_ERR_STATE once an engine has reallocated the buffers the graph uses
 * (a later solve with more right-hand sides, another set of coefficients).
 * Destroy graphs before their engines.  Replaces, per engine, the host-driven
 * loop of Domain_Solver.solve (src_solver/slablu_solver.py:543-600 sweeps
 * solve_slab and Tred_solver.solve once per call); the reference has no
 * multi-problem launch.
 */
typedef struct slab_solve_graph slab_solve_graph;
int slab_solve_graph_create(slab_solve_graph** out, slab_engine* const* engines, int count, const int* nrhs,
                            const double* const* d_bnd, const double* const* d_fbody, double* const* d_uleaf,
                            double tol, int max_iter);
/* Launch on `stream` (cudaStream_t; NULL = legacy stream): ordered after all
 * earlier work of the engines and before their later work; asynchronous. */
int slab_solve_graph_launch(slab_solve_graph* g, void* stream);
/* Waits for the last launch; h_iters / h_stats (5 doubles, as for
 * slab_engine_solve) of engine i.  SLAB_ERR_NOCONV if it did not reach tol. */
int slab_solve_graph_status(slab_solve_graph* g, int i, int* h_iters, double* h_stats);
int slab_solve_graph_destroy(slab_solve_graph* g);

/* FP64 residual of the full HPS collocation system at (u_faces, u_int):
 * r_int = f - Aloc[Jc,:] u per leaf, r_faces = -sum of leaf fluxes Nx u at
 * interior faces (nfaces x nrhs column-major; zero on Dirichlet faces).
 * d_uint / d_rint: interior values leaf-major, element (leaf, rhs c, interior
 * node r) at (leaf*nrhs + c)*(p-2)^2 + r.  d_fbody as for slab_engine_solve. */
int slab_engine_residual(slab_engine* e, int nrhs, const double* d_ufaces, const double* d_uint,
                         const double* d_fbody, double* d_rint, double* d_rfaces);

/* One application of the stored factorization to a residual: the correction
 * (d_dint, d_dfaces) = M^-1 (d_rint, d_rfaces) that one refinement step of
 * slab_engine_solve adds, with M the factorization in the engine's precision
 * (leaf, merge-tree and interface sweeps).  Layouts as for slab_engine_residual;
 * d_rfaces entries on Dirichlet faces are read as zero and d_dfaces is zero
 * there.  For callers that drive their own iteration (a Krylov method with the
 * factorization as preconditioner).  The reference applies its factorization
 * only inside solve (src_solver/slablu_solver.py:543-666). */
int slab_engine_apply(slab_engine* e, int nrhs, const double* d_rint, const double* d_rfaces, double* d_dint,
                      double* d_dfaces);

/* Adjoint (transposed) solve with the stored factors, for the gradient of a
 * loss L(u) through slab_engine_solve.  Extends Domain_Solver.solve
 * (src_solver/slablu_solver.py:623-666); the transposed pieces follow
 * lusolve_sweep_transpose (src_solver/block_tridiag_solver_dense.py:205-222)
 * and solve_slab(transpose=True) (src_solver/slablu_solver.py:901-943).
 *   d_gleaf  : dL/du at every leaf node (nleaves*p*p x nrhs column-major), or NULL
 *   d_gfaces : dL/du_faces (nfaces x nrhs column-major), or NULL
 * Solves A^T lam = g on the full collocation system with FP64 refinement (same
 * tol / max_iter meaning as slab_engine_solve) and writes, each optional:
 *   d_lam_leaf  : multipliers of the interior PDE rows at the leaf nodes
 *                 (zero on leaf boundary nodes) = dL/d(body load)
 *   d_lam_faces : multipliers of the face flux rows (zero on Dirichlet faces)
 *   d_gbnd      : dL/d(Dirichlet data) on Dirichlet faces, zero elsewhere
 *                 (nfaces x nrhs, the layout of slab_engine_solve's d_bnd).
 * Leaf order and merge blocks are limited to 512 unknowns (p <= 24 with the
 * default slab widths).  h_stats as for slab_engine_solve (worst column). */
int slab_engine_adjoint(slab_engine* e, int nrhs, const double* d_gleaf, const double* d_gfaces, double tol,
                        int max_iter, double* d_lam_leaf, double* d_lam_faces, double* d_gbnd, int* h_iters,
                        double* h_stats);

/* Gradient of L with respect to the PDE coefficient fields at the leaf nodes,
 * summed over the nrhs columns: d_g* (nleaves*p*p each, NULL to skip) from the
 * forward solution (d_ufaces, d_uleaf of slab_engine_solve) and d_lam_leaf of
 * slab_engine_adjoint.  dL/dc = -lam*u, dL/dc11 = lam*(D11 u), dL/dc22 =
 * lam*(D22 u), dL/dc1 = -lam*(D1 u), dL/dc2 = -lam*(D2 u) at interior nodes,
 * zero at leaf boundary nodes (which carry no PDE row); Aloc as in
 * src_disc/hps_parallel_leaf_ops.py:17-27. */
int slab_engine_coeff_grad(slab_engine* e, int nrhs, const double* d_ufaces, const double* d_uleaf,
                           const double* d_lam_leaf, double* d_gc11, double* d_gc22, double* d_gc1, double* d_gc2,
                           double* d_gc);

/* The same for an engine from slab_engine_create_mixed, with dL/dc12 in d_gc12
 * (NULL to skip): every term is evaluated on the node values the PDE rows see,
 * the interior values and Interp_mat u_faces on the leaf boundary (corners
 * included), and dL/dc12 = 2 lam (D12 u) with D12 = kron(D, D) (the c12 term
 * -2 c12 D12 of Aloc, src_disc/hps_parallel_leaf_ops.py:17-27).  On an engine
 * without c12 a non-NULL d_gc12 returns SLAB_ERR_ARG; slab_engine_coeff_grad on
 * a mixed engine gives the other five. */
int slab_engine_coeff_grad_mixed(slab_engine* e, int nrhs, const double* d_ufaces, const double* d_uleaf,
                                 const double* d_lam_leaf, double* d_gc11, double* d_gc22, double* d_gc12,
                                 double* d_gc1, double* d_gc2, double* d_gc);

/* FP64 matrix product on the BF16 tensor cores (tcgen05) by exact slicing:
 * C = alpha A B + beta C with A (m x k), B (k x n), C (m x n), column-major
 * device arrays.  Rows of A and columns of B are scaled by powers of two, cut
 * into eight 7-bit integer slices and multiplied with exact FP32 accumulation;
 * the error is bounded by about k 2^-53 max|A(i,:)| max|B(:,j)| per entry.
 * Non-finite inputs give NaN in the affected rows/columns.  d_work: at least
 * slab_dgemm_emu_work_bytes(m, n, k) bytes.  Synchronizes the stream to report
 * failures.  No counterpart in the reference (used inside the interface
 * factorization, block_tridiag_solver_structured.py:34-76). */
size_t slab_dgemm_emu_work_bytes(int m, int n, int k);
int slab_dgemm_emu(int m, int n, int k, double alpha, const double* d_A, int lda, const double* d_B, int ldb,
                   double beta, double* d_C, int ldc, void* d_work, size_t work_bytes, void* stream);

/* Batched FP32 matrix product on the TF32 tensor cores (tcgen05) by exact
 * three-way TF32 splitting: C[b] = alpha A[b] B[b] + beta C[b] for b < batch,
 * A (m x k), B (k x n), C (m x n) column-major device arrays with batch strides
 * in elements.  Each operand is split into three TF32 values summing to it
 * exactly and the six slice products of weight down to 2^-22 are accumulated
 * in FP32 in tensor memory: the error stays within the FP32 dot-product bound
 * k 2^-24 max|A(i,:)| max|B(:,j)|.  C may alias B.  d_work: at least
 * 256 + slab_sgemm_tc_work_bytes(m, n, k, batch) bytes, 256-byte aligned.
 * Synchronizes the stream to report failures.  Replaces the batched products
 * of the slab Schur arithmetic (the Schur update T_i - L U of
 * src_solver/block_tridiag_solver_dense.py:169 and the slab interface products
 * of src_solver/slablu_solver.py:1066-1136), which the engine calls
 * asynchronously inside its factorization. */
/* Dense FP64 LU with partial pivoting of one n x n column-major device matrix
 * (in place, L unit-lower and U) with the library's FP64 panel and update
 * kernels, and solves with it.  d_work (slab_dense_lu_work_bytes(n) bytes,
 * 256-byte aligned) keeps the pivots and the inverted 64-row diagonal blocks
 * between the two calls.  slab_dense_lu returns the LAPACK info of the first
 * zero pivot (> 0) and also writes it to *h_info (may be NULL); it synchronizes
 * the stream.  slab_dense_lu_solve: X = A^{-1} B (n x nrhs, X != B),
 * asynchronous.  Replaces the lu_factor / lu_solve of the periodic interface
 * Schur complement (src_solver/block_tridiag_solver_structured.py:118-154,
 * 193-206), used by the periodic edge (slablu_gb300/periodic.py). */
size_t slab_dense_lu_work_bytes(int n);
int slab_dense_lu(int n, double* d_A, int lda, void* d_work, size_t work_bytes, int* h_info, void* stream);
int slab_dense_lu_solve(int n, int nrhs, const double* d_LU, int lda, const void* d_work, const double* d_B, int ldb,
                        double* d_X, int ldx, void* stream);

size_t slab_sgemm_tc_work_bytes(int m, int n, int k, int batch);
int slab_sgemm_tc(int m, int n, int k, float alpha, const float* d_A, int lda, long long strideA, const float* d_B,
                  int ldb, long long strideB, float beta, float* d_C, int ldc, long long strideC, int batch,
                  void* d_work, size_t work_bytes, void* stream);

/*
 * Reduced sparse operator on the device (CSR, FP64).
 * Replaces the COO -> CSR assembly of HPS_Multidomain.sparse_mat
 * (src_disc/hps_multidomain_disc.py:53-109: the leaf DtN maps summed over the
 * reduced face unknowns) and the sparse applies of the right-hand-side
 * formation (src_solver/slablu_solver.py:48-57 apply_sparse_lowmem, :489-507
 * get_rhs).  The pattern depends only on the leaf grid and is built on the host
 * (slablu_gb300/sparse.py); d_dest maps every leaf DtN entry (leaf-major,
 * row-major within a leaf) to its CSR slot.
 *   slab_csr_assemble: d_vals[0..nnz) = 0, then d_vals[d_dest[i]] += d_src[i]
 *                      for i < count (at most two terms per slot: the sum is
 *                      independent of their order).
 *   slab_csr_spmv:     d_y = alpha A d_x + beta d_y for the nrows x ncols CSR
 *                      matrix (d_indptr nrows+1 64-bit offsets, d_indices int32).
 */
int slab_csr_assemble(long long count, const double* d_src, const long long* d_dest, long long nnz,
                      double* d_vals, void* stream);
int slab_csr_spmv(int nrows, const long long* d_indptr, const int* d_indices, const double* d_vals,
                  const double* d_x, double alpha, double beta, double* d_y, void* stream);

/* Tunable launch choices of an engine (slablu_gb300/autotune.py times them):
 *   SLAB_OPT_LEAF_CTAS   resident leaves per SM in the leaf kernel, 0 = as many
 *                        as fit (fewer keep more of each leaf matrix in L2)
 *   SLAB_OPT_IFACE_SOLVE interface triangular solves: 0 one thread-block cluster,
 *                        1 grid-wide cooperative kernel
 *   SLAB_OPT_IFACE_LOOKAHEAD interface block LU (mixed and fp32 engines): 1
 *                        overlaps each 256-column outer block's update of the
 *                        columns beyond the next block with that block's panels
 *                        (second stream), 0 serial; both give the same factors
 *   SLAB_OPT_TREE_TC     FP32 merge tree (mixed and fp32 engines): 1 forms the
 *                        merges' Schur updates F -= col W as TF32-split
 *                        tensor-core products (slab_sgemm_tc), 0 on the CUDA
 *                        cores; fp64 engines accept 0 only
 *   SLAB_OPT_LEAF_ASSEMBLY leaf operators without c12: 1 assembled by a kernel
 *                        of their own at full occupancy before the factor
 *                        kernel, 0 inside the factor kernel; same factors
 *   SLAB_OPT_IFACE_OUTER_INV interface block LU (mixed precision): 1 applies
 *                        S_j^{-1} to the Schur right-hand sides through inverted
 *                        256-row diagonal blocks of L and U, every product on the
 *                        tensor cores; 0 solves inside each 256-row block with
 *                        FP64-core triangular solves of 64-row blocks
 *   SLAB_OPT_IFACE_PANEL interface block LU (fp32 engines): 0 factors each
 *                        32-column pivoted panel of up to 1536 rows in one CTA
 *                        (one block barrier per column; taller panels in a
 *                        cluster), 1 every panel in a thread-block cluster (one
 *                        cluster barrier per column); same pivots and factors
 *   SLAB_OPT_GEMM_TILES  FP32 products (merge tree, FP32 interface): 0 128 x 128
 *                        output tiles where their grid fills the GPU, 64 x 64
 *                        otherwise; 1 always 64 x 64; same sums in the same order
 * set returns a status; get returns the value (or a negative status). */
#define SLAB_OPT_LEAF_CTAS 1
#define SLAB_OPT_IFACE_SOLVE 2
#define SLAB_OPT_IFACE_LOOKAHEAD 3
#define SLAB_OPT_TREE_TC 4
#define SLAB_OPT_LEAF_ASSEMBLY 5
#define SLAB_OPT_IFACE_OUTER_INV 6
#define SLAB_OPT_IFACE_PANEL 7
#define SLAB_OPT_GEMM_TILES 8
int slab_engine_set_option(slab_engine* e, int key, int value);
int slab_engine_get_option(const slab_engine* e, int key);

/* Bytes of device memory held by the engine's factorization. */
size_t slab_engine_factor_bytes(const slab_engine* e);

/* Bytes of stored factors one solve application reads (leaf LU and S, merge
 * factors, the interface factors applied in the solve phase, pivots): the
 * algorithmic traffic of the memory-bound solve sweep.  The reference reads
 * its factors in lusolve_sweep and __solve_lowmem
 * (src_solver/block_tridiag_solver_dense.py:179-202,
 * src_solver/block_tridiag_solver_structured.py:157-187). */
size_t slab_engine_solve_bytes(const slab_engine* e);

/* Device times (CUDA events on the engine stream, milliseconds) of the last
 * factor and solve: [0] leaf kernel, [1] slab merge tree, [2] interface block
 * LU, [3] whole solve, [4] sum of the factorization applications inside the
 * solve, [5] number of those applications.  Writes min(n, 6) values and
 * returns that count. */
int slab_engine_timings(const slab_engine* e, double* h_ms, int n);

/* Number of kernel launches issued by the library since it was loaded. */
long long slab_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* SLABLU_GB300_H */
