"""Oracle: batched block-tridiagonal LU sweeps (test infrastructure only).

Restates, in NumPy/SciPy and FP64,
  src_solver/block_tridiag_solver_dense.py:111-140  solveU / solveL (fast_LU=False)
  src_solver/block_tridiag_solver_dense.py:152-177  build_sweep
  src_solver/block_tridiag_solver_dense.py:179-202  lusolve_sweep
  src_solver/block_tridiag_solver_dense.py:205-222  lusolve_sweep_transpose
  src_solver/block_tridiag_solver_dense.py:468-488  matvec / matvec_transpose
  src_solver/block_tridiag_solver_structured.py:34-76, 157-187
                                                     interface block LU (build_lowmem_helper,
                                                     __solve_lowmem) on dense blocks
  src_solver/block_tridiag_solver_structured.py:118-154, 189-206
                                                     cyclic interface system (periodic
                                                     boundary): corner block eliminated last
Pivot vectors are LAPACK's (0-based here, 1-based in torch); the factor
values are identical to the reference's because both call getrf.
"""
import numpy as np
import scipy.linalg as sla


def _lu(A):
    return sla.lu_factor(A, check_finite=False)


def _L_solve(lu, piv, B):
    """L^{-1} P^T B: apply the row interchanges, then the unit lower solve."""
    X = np.array(B, dtype=float, copy=True)
    for i, pi in enumerate(piv):
        if pi != i:
            X[[i, pi]] = X[[pi, i]]
    return sla.solve_triangular(lu, X, lower=True, unit_diagonal=True, check_finite=False)


def _U_solve(lu, B, trans=False):
    return sla.solve_triangular(lu, B, lower=False, trans=1 if trans else 0, check_finite=False)


def _Lt_solve(lu, piv, B):
    """P L^{-T} B."""
    X = sla.solve_triangular(lu, B, lower=True, unit_diagonal=True, trans=1, check_finite=False)
    for i in range(len(piv) - 1, -1, -1):
        pi = piv[i]
        if pi != i:
            X[[i, pi]] = X[[pi, i]]
    return X


class BlockTridiag:
    """Batched block-tridiagonal LU with partial pivoting inside diagonal blocks.

    diag: (b, m, bs, bs); sub: (b, m-1, bs, bs) = A[i+1, i]; sup: (b, m-1, bs, bs) = A[i, i+1].
    After construction: LU/piv of the Schur diagonal blocks, Lsub = sub U^{-1},
    Usup = L^{-1} P^T sup (build_sweep, block_tridiag_solver_dense.py:152-177).
    """

    def __init__(self, diag, sub, sup):
        self.b, self.m, self.bs = diag.shape[0], diag.shape[1], diag.shape[2]
        b, m = self.b, self.m
        self.diag0, self.sub0, self.sup0 = diag.copy(), sub.copy(), sup.copy()
        self.LU = np.empty_like(diag)
        self.piv = np.empty((b, m, self.bs), dtype=np.int64)
        self.Lsub = np.empty_like(sub)
        self.Usup = np.empty_like(sup)
        for k in range(b):
            lu, pv = _lu(diag[k, 0])
            self.LU[k, 0], self.piv[k, 0] = lu, pv
            for i in range(1, m):
                Uf = _L_solve(lu, pv, sup[k, i - 1])
                Lf = _U_solve(lu, sub[k, i - 1].T, trans=True).T
                lu, pv = _lu(diag[k, i] - Lf @ Uf)
                self.LU[k, i], self.piv[k, i] = lu, pv
                self.Usup[k, i - 1], self.Lsub[k, i - 1] = Uf, Lf

    def solve(self, f, b_start=0, b_end=None, transpose=False):
        """f: (nb, m*bs, nrhs) -> solution (lusolve_sweep / _transpose)."""
        b_end = self.b if b_end is None else b_end
        m, bs = self.m, self.bs
        nb, _, nrhs = f.shape
        F = f.reshape(nb, m, bs, nrhs).astype(float).copy()
        for kk in range(nb):
            k = b_start + kk
            LU, pv, Ls, Us = self.LU[k], self.piv[k], self.Lsub[k], self.Usup[k]
            x = F[kk]
            if not transpose:
                x[0] = _L_solve(LU[0], pv[0], x[0])
                for i in range(1, m):
                    x[i] = _L_solve(LU[i], pv[i], x[i] - Ls[i - 1] @ x[i - 1])
                x[m - 1] = _U_solve(LU[m - 1], x[m - 1])
                for i in range(m - 2, -1, -1):
                    x[i] = _U_solve(LU[i], x[i] - Us[i] @ x[i + 1])
            else:
                x[0] = _U_solve(LU[0], x[0], trans=True)
                for i in range(1, m):
                    x[i] = _U_solve(LU[i], x[i] - Us[i - 1].T @ x[i - 1], trans=True)
                x[m - 1] = _Lt_solve(LU[m - 1], pv[m - 1], x[m - 1])
                for i in range(m - 2, -1, -1):
                    x[i] = _Lt_solve(LU[i], pv[i], x[i] - Ls[i].T @ x[i + 1])
        return F.reshape(nb, m * bs, nrhs)

    def matvec(self, u, transpose=False):
        """Apply the original block-tridiagonal operator (block_tridiag_solver_dense.py:468-488)."""
        b, m, bs = self.b, self.m, self.bs
        U = u.reshape(b, m, bs, -1)
        F = np.zeros_like(U)
        t = (lambda M: np.swapaxes(M, -1, -2)) if transpose else (lambda M: M)
        for i in range(m):
            F[:, i] += t(self.diag0[:, i]) @ U[:, i]
        for i in range(m - 1):
            if not transpose:
                F[:, i + 1] += self.sub0[:, i] @ U[:, i]
                F[:, i] += self.sup0[:, i] @ U[:, i + 1]
            else:
                F[:, i] += t(self.sub0[:, i]) @ U[:, i + 1]
                F[:, i + 1] += t(self.sup0[:, i]) @ U[:, i]
        return F.reshape(b, m * bs, -1)


class InterfaceBlockLU:
    """Sequential interface block LU over dense blocks.

    S_0 = diag_0 ;  S_j = diag_j - sub_{j-1} S_{j-1}^{-1} sup_{j-1}
    (block_tridiag_solver_structured.py:34-76), solved by the forward/backward
    sweep of :157-187.  diag: (nb, n, n); sub/sup: (nb-1, n, n).
    """

    def __init__(self, diag, sub, sup):
        self.nb, self.n = diag.shape[0], diag.shape[1]
        self.sub, self.sup = sub, sup
        self.LU, self.piv = [], []
        lu, pv = _lu(diag[0])
        self.LU.append(lu); self.piv.append(pv)
        for j in range(1, self.nb):
            S = diag[j] - sub[j - 1] @ sla.lu_solve((lu, pv), sup[j - 1], check_finite=False)
            lu, pv = _lu(S)
            self.LU.append(lu); self.piv.append(pv)

    def solve(self, f):
        F = np.array(f, dtype=float, copy=True)
        nb = self.nb
        F[0] = _L_solve(self.LU[0], self.piv[0], F[0])
        for j in range(nb - 1):
            t = _U_solve(self.LU[j], F[j])
            F[j + 1] = _L_solve(self.LU[j + 1], self.piv[j + 1], F[j + 1] - self.sub[j] @ t)
        F[nb - 1] = _U_solve(self.LU[nb - 1], F[nb - 1])
        for j in range(nb - 2, -1, -1):
            t = _L_solve(self.LU[j], self.piv[j], self.sup[j] @ F[j + 1])
            F[j] = _U_solve(self.LU[j], F[j] - t)
        return F


class CyclicInterfaceBlockLU:
    """Cyclic block-tridiagonal interface system of a periodic domain.

    Block j couples to j-1 and j+1 modulo nb: sub[j] is block (j, j-1 mod nb)
    and sup[j] is block (j, j+1 mod nb); diag, sub, sup are (nb, n, n).  As in
    block_tridiag_solver_structured.py:118-154, blocks 1..nb-1 form an acyclic
    system (factored by InterfaceBlockLU), the two couplings of block 0 are
    carried through it, V = A'^{-1} [-sub_1; 0; ...; 0; -sup_{nb-1}], and the
    Schur complement of block 0, X = diag_0 + sup_0 V_0 + sub_0 V_{nb-2}, is
    LU-factored.  The solve (:189-206): u = A'^{-1} f[1:], x_0 = X^{-1}
    (f_0 - sup_0 u_0 - sub_0 u_{nb-2}), x[1:] = V x_0 + u.
    """

    def __init__(self, diag, sub, sup):
        nb, n = diag.shape[0], diag.shape[1]
        if nb < 3:
            raise ValueError('a cyclic interface system needs at least 3 blocks')
        self.nb, self.n = nb, n
        self.inner = InterfaceBlockLU(diag[1:], sub[2:], sup[1:nb - 1])
        W = np.zeros((nb - 1, n, n))
        W[0] = -sub[1]
        W[nb - 2] = -sup[nb - 1]
        self.V = self.inner.solve(W)
        X = diag[0] + sup[0] @ self.V[0] + sub[0] @ self.V[nb - 2]
        self.X = _lu(X)
        self.sub0, self.sup0 = sub[0], sup[0]

    def solve(self, f):
        """f: (nb, n, nrhs) -> (nb, n, nrhs)."""
        F = np.asarray(f, dtype=float)
        u = self.inner.solve(F[1:])
        rhs = F[0] - self.sup0 @ u[0] - self.sub0 @ u[self.nb - 2]
        out = np.empty_like(F)
        out[0] = sla.lu_solve(self.X, rhs, check_finite=False)
        out[1:] = np.einsum('kij,jr->kir', self.V, out[0]) + u
        return out
