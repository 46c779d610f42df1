// FP64 matrix products on the BF16 tensor cores by exact slicing (ozaki.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace slab {

// Work bytes of dgemm_emu for an (m x k) (k x n) product.
size_t dgemm_emu_work_bytes(int m, int n, int k);

// C = alpha A B + beta C (column-major FP64) on the tensor cores; asynchronous
// on stream s.  work: dgemm_emu_work_bytes(m, n, k) bytes whose first 256 are
// left to the caller; err: device int, set nonzero if a pipeline wait expired
// (C is then not written).
int dgemm_emu(cudaStream_t s, int m, int n, int k, double alpha, const double* A, int lda, const double* B, int ldb,
              double beta, double* C, int ldc, void* work, size_t work_bytes, int* err);

// Workspace of the blocked routines below: dgemm_emu work plus its error flag.
struct EmuWork {
  void* buf = nullptr;
  size_t bytes = 0;
  int* err = nullptr;
};

// Outer block of the blocked routines: products of this depth go to dgemm_emu,
// the work inside an outer block stays on the FP64 cores.
constexpr int kEmuOuter = 256;

// bigtrs_inv (X = U^{-1} L^{-1} P B, inverted bs x bs diagonal triangles) with
// the updates between outer blocks of kEmuOuter rows done by dgemm_emu.
int bigtrs_inv_emu(cudaStream_t s, const double* LU, int lda, int n, const int* perm, const double* Linv,
                   const double* Uinv, int bs, const double* B, int ldb, double* X, int ldx, int nrhs,
                   const EmuWork& w);

// Inverses of the kEmuOuter-row diagonal blocks of the unit-lower L and the
// upper U of an n x n LU (column-major, lda), built from the inverses of their
// 64-row diagonal blocks (tri_inv_blocks layout: block k at Linv64 + k*64*64,
// ld 64, zero outside its triangle) by two doubling steps on the FP64 cores:
//   [[A, 0], [B, C]]^{-1} = [[A^{-1}, 0], [-C^{-1} B A^{-1}, C^{-1}]]
//   [[A, B], [0, C]]^{-1} = [[A^{-1}, -A^{-1} B C^{-1}], [0, C^{-1}]].
// LoInv / UoInv: ceil(n / kEmuOuter) blocks of kEmuOuter x kEmuOuter (ld
// kEmuOuter, zero outside the triangle); tmp: outer_tri_tmp_elems(n) doubles.
size_t outer_tri_tmp_elems(int n);
int outer_tri_inverses(cudaStream_t s, const double* LU, int lda, int n, const double* Linv64, const double* Uinv64,
                       double* LoInv, double* UoInv, double* tmp);

// X = U^{-1} L^{-1} P B with the outer-block inverses of outer_tri_inverses:
// per outer block one tensor-core product with the inverted diagonal block
// (through Y, kEmuOuter x nrhs doubles) and one with the off-diagonal rows, all
// by dgemm_emu (no FP64-core triangular solves).
int bigtrs_outer_emu(cudaStream_t s, const double* LU, int lda, int n, const int* perm, const double* LoInv,
                     const double* UoInv, const double* B, int ldb, double* X, int ldx, int nrhs, double* Y,
                     const EmuWork& w);

// Second stream for the lookahead of biglu_emu.  side == null: serial.
struct Lookahead {
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  int* perm = nullptr;  // 1 + 2 * kRowpermMax ints (row-interchange gather)
};

// biglu with the trailing update between outer blocks of kEmuOuter columns
// done by dgemm_emu (the panels and the updates inside an outer block stay on
// the FP64 cores).  Same pivots, factors and info as biglu.  panel_linv: kNB x
// kNB doubles; blk_linv: kEmuOuter * 64 doubles.
// With la->side, each outer block's update of the columns beyond the next
// outer block runs on the side stream while the next outer block's panels
// are factored on s: panel interchanges are applied inside the outer block at
// once and to the other columns after the block (as one gather), once the
// side stream no longer reads them.  The result is the same.
int biglu_emu(cudaStream_t s, double* A, int lda, int n, int* ipiv, int* info, double* panel_linv, double* blk_linv,
              const EmuWork& w, const Lookahead* la = nullptr);

}  // namespace slab
