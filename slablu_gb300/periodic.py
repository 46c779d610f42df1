"""Periodic boundary in x: the left and right edges of the rectangle are one curve.

Mirrors Domain_Solver(periodic_bc=True) of src_solver/slablu_solver.py: the
index sets of the periodic partition (:89-120), the folded right-hand side and
residual (:489-541) and the periodic solve (:543-599, 623-666), where Dirichlet
data is given on the bottom and top faces only and the shared edge (the left
edge of slab 0, the right edge of the last slab) is unknown.

The reference eliminates the shared edge inside a cyclic interface system
(src_solver/block_tridiag_solver_structured.py:118-154, 189-206).  Here the
factorization of the GPU engine is the non-periodic one (both edge copies are
Dirichlet faces), and the edge is coupled back through its Schur complement:
with U_k the engine solution for unit data on both copies of edge node k (zero
elsewhere), and the flux balance at the edge

    r(u) = (A u)[left edge] + (A u)[right edge]        (A: reduced operator),

the edge values y of the periodic solution solve S y = -r(u_0), S[:, k] = r(U_k),
where u_0 is the engine solution with the edge set to zero.  Then one engine
solve with y on both copies gives the periodic solution (the map from edge data
to solution is linear); a few correction steps S dy = -r(u) take it to the
engine's FP64 accuracy.  Building S costs one engine solve column per edge node
(n1 (p-2) columns, done in chunks) and one dense LU of n1 (p-2) unknowns.
"""
import ctypes

import numpy as np
import torch

from . import _lib


def periodic_index_sets(geom):
    """The reference's periodic index sets (slablu_solver.py:89-120) on a Geometry.

    I_slabX: every slab's left edge, then the last slab's right edge; I_Xtot:
    the bottom and top faces; I_Ctot = [I_slabC, I_slabX]; within I_Ctot,
    I_Ctot_copy1 is slab 0's left edge, I_Ctot_copy2 the last slab's right edge
    (its copy, last), I_Ctot_unique everything but copy2.
    """
    ip = geom.inds_pans
    nL, nC, npan = geom.I_L.size, geom.I_C.size, geom.Npan
    I_slabX = np.concatenate((ip[:, geom.I_L].ravel(), ip[-1, geom.I_R]))
    I_slabC = ip[:, geom.I_C].ravel()
    off = nC * npan
    return dict(I_slabC=I_slabC, I_slabX=I_slabX, I_Ctot=np.concatenate((I_slabC, I_slabX)),
                I_Xtot=np.concatenate((ip[:, geom.I_D].ravel(), ip[:, geom.I_U].ravel())),
                I_Ctot_unique=np.arange(off + nL * npan), I_Ctot_copy1=np.arange(nL) + off,
                I_Ctot_copy2=np.arange(nL) + off + nL * npan)


def edge_faces(geom):
    """Reduced indices of the two copies of the shared edge: (left of slab 0, right of the last slab)."""
    return geom.inds_pans[0, geom.I_L], geom.inds_pans[-1, geom.I_R]


def fold(v, sets):
    """Rows of a vector on the periodic I_Ctot folded onto the unique unknowns:
    the right-edge copy added to the left edge (slablu_solver.py:520-524)."""
    c1 = torch.as_tensor(sets['I_Ctot_copy1'], device=v.device)
    c2 = torch.as_tensor(sets['I_Ctot_copy2'], device=v.device)
    u = torch.as_tensor(sets['I_Ctot_unique'], device=v.device)
    out = v.clone()
    out[c1] += v[c2]
    return out[u]


class DenseLU:
    """FP64 LU with partial pivoting of a square CUDA matrix and solves with it,
    by the library's FP64 kernels (slab_dense_lu / slab_dense_lu_solve)."""

    def __init__(self, S):
        if not S.is_cuda:
            raise ValueError('DenseLU factors CUDA matrices (slablu_gb300 has no CPU path)')
        L = _lib.lib()
        self.n = S.shape[0]
        self.LU = S.T.contiguous().to(torch.float64)       # column-major storage
        self.wb = int(L.slab_dense_lu_work_bytes(self.n))
        self.work = torch.empty(self.wb, dtype=torch.uint8, device=S.device)
        info = ctypes.c_int(0)
        st = L.slab_dense_lu(self.n, _lib.ptr(self.LU), self.n, _lib.ptr(self.work), ctypes.c_size_t(self.wb),
                             ctypes.byref(info), _stream(S.device))
        _lib.check(st, 'slab_dense_lu')

    def solve(self, B):
        """A^{-1} B for B (n,) or (n, k)."""
        L = _lib.lib()
        B2 = B if B.dim() == 2 else B[:, None]
        Bc = B2.T.contiguous().to(torch.float64)
        X = torch.empty_like(Bc)
        st = L.slab_dense_lu_solve(self.n, Bc.shape[0], _lib.ptr(self.LU), self.n, _lib.ptr(self.work),
                                   _lib.ptr(Bc), self.n, _lib.ptr(X), self.n, _stream(B.device))
        _lib.check(st, 'slab_dense_lu_solve')
        X = X.T
        return X if B.dim() == 2 else X[:, 0]


def _stream(dev):
    return ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


class PeriodicEdge:
    """Schur complement of the shared edge on top of a non-periodic factorization.

    ``engine`` has the interface of SlabEngine.solve(bnd, fbody, tol, max_iter,
    want_faces, allow_noconv, want_leaf) -> (u_leaf, u_faces, iters, stats), with
    both edge copies among its Dirichlet faces; ``edge_flux(u_faces)`` returns the
    reduced operator's rows at [left edge; right edge] applied to face vectors
    (ntot, k).  Only the final solve asks for the leaf-node solution.
    """

    def __init__(self, engine, edge_flux, left, right, ntot, tol=1e-10, max_iter=20, chunk=128, dense_lu=DenseLU):
        self.engine, self.edge_flux = engine, edge_flux
        self.dense_lu = dense_lu   # factorization of the edge Schur complement: DenseLU(S).solve(B)
        self.ntot, self.tol, self.max_iter = int(ntot), tol, max_iter
        self.nL = len(left)
        if len(right) != self.nL:
            raise ValueError('the two edge copies must have the same length')
        self.dev = None
        self._left_np, self._right_np = np.asarray(left), np.asarray(right)
        self.chunk = max(1, int(chunk))
        self.S = None

    def _idx(self, dev):
        return (torch.as_tensor(self._left_np, device=dev), torch.as_tensor(self._right_np, device=dev))

    def _solve_faces(self, bnd, fbody=None, want_leaf=True):
        return self.engine.solve(bnd, fbody, tol=self.tol, max_iter=self.max_iter, want_faces=True,
                                 allow_noconv=True, want_leaf=want_leaf)

    def _residual(self, uf):
        f = self.edge_flux(uf)
        return f[:self.nL] + f[self.nL:]

    def build(self, dev):
        """S[:, k] = r(U_k), in chunks of unit-data columns."""
        self.dev = torch.device(dev)
        L, R = self._idx(self.dev)
        nL = self.nL
        S = torch.empty(nL, nL, dtype=torch.float64, device=self.dev)
        self.build_iters = 0
        for c0 in range(0, nL, self.chunk):
            k = min(self.chunk, nL - c0)
            bnd = torch.zeros(self.ntot, k, dtype=torch.float64, device=self.dev)
            cols = torch.arange(k, device=self.dev)
            bnd[L[c0:c0 + k], cols] = 1.0
            bnd[R[c0:c0 + k], cols] = 1.0
            _, uf, iters, _ = self._solve_faces(bnd, want_leaf=False)
            self.build_iters = max(self.build_iters, iters)
            S[:, c0:c0 + k] = self._residual(uf)
        self.S = S
        self.lu = self.dense_lu(S)
        return self

    def solve(self, bnd, fbody=None, max_refine=4):
        """Periodic solve.  bnd (ntot, k): Dirichlet data on the bottom and top faces
        (values on the edge copies are ignored).  Returns (u_leaf, u_faces, stats)
        where stats holds the engine's last stats, the edge correction steps and the
        relative edge residual."""
        if self.S is None:
            raise RuntimeError('PeriodicEdge.build() first')
        if fbody is not None:
            # the edge flux balance is formed from the face values alone (edge_flux); a
            # body load adds its particular flux at the edge, which that map leaves out
            raise NotImplementedError('PeriodicEdge.solve: body loads with periodic boundaries')
        L, R = self._idx(bnd.device)
        b = bnd.clone()
        if b.dim() == 1:
            b = b[:, None]
        b[L] = 0.0
        b[R] = 0.0
        _, uf, iters, st = self._solve_faces(b, fbody, want_leaf=False)
        r0 = self._residual(uf)
        y = -self.lu.solve(r0)
        steps, total_iters = 0, iters
        r0n = float(torch.linalg.norm(r0))
        while True:
            b[L] = y
            b[R] = y
            uleaf, uf, iters, st = self._solve_faces(b, fbody)
            total_iters += iters
            steps += 1
            r = self._residual(uf)
            rn = float(torch.linalg.norm(r))
            dy = -self.lu.solve(r)
            yn = float(torch.linalg.norm(y))
            if steps >= max_refine or yn == 0.0 or float(torch.linalg.norm(dy)) <= self.tol * yn:
                break
            y = y + dy
        stats = dict(st, edge_steps=steps, engine_iters=total_iters,
                     edge_rel_residual=(rn / r0n if r0n > 0 else 0.0))
        return uleaf, uf, stats
