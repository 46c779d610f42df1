"""Oracle: the finite-difference discretisation and its slab partition (test infrastructure only).

Restates, in NumPy/SciPy and FP64,
  src_disc/fd_disc.py:12-27     get_inds_2d
  src_disc/fd_disc.py:50-81     grid (2-D)
  src_disc/fd_disc.py:83-140    FD_disc (2-D five-point operator, assemble_sparse)
  src_solver/slablu_solver.py:212-296  fd_panel_split (slab widths, index sets, I_C order)
  src_solver/slablu_solver.py:83-120   the FD branch of Domain_Solver.__init__ (I_Ctot, I_Xtot)
The solve is the superLU black-box path of oracle/domain.py on these index sets.
The reference's first-order y term is broken (fd_disc.py:133-138 reads c1 and an
undefined D1), so an operator with c2 is rejected here.
"""
import numpy as np
import scipy.sparse as sp

from .domain import nearest_divisor


def _arange_like_torch(start, stop, step):
    """The reference's grid axis, torch.arange in float64 (its points can differ from
    start + i step in the last bit, so the axis is taken from torch itself)."""
    import torch
    return torch.arange(float(start), float(stop), float(step), dtype=torch.float64).numpy()


def grid(box_geom, h):
    """Grid points (2, n0 n1), x-major (fd_disc.py:50-67), and (n0, n1)."""
    box = np.asarray(box_geom, dtype=float)
    xx0 = _arange_like_torch(box[0, 0], box[0, 1] + 0.5 * h, h)
    xx1 = _arange_like_torch(box[1, 0], box[1, 1] + 0.5 * h, h)
    n0, n1 = xx0.size, xx1.size
    XX = np.vstack((np.repeat(xx0, n1), np.tile(xx1, n0)))
    return XX, n0, n1


def boundary_indices(XX, box_geom, h):
    """I_L, I_R (without the bottom and top rows) and I_DIR (bottom and top), :12-27."""
    box = np.asarray(box_geom, dtype=float)
    I_L = np.flatnonzero(XX[0] < 0.5 * h + box[0, 0])
    I_R = np.flatnonzero(XX[0] > -0.5 * h + box[0, 1])
    I_D = np.flatnonzero(XX[1] < 0.5 * h + box[1, 0])
    I_U = np.flatnonzero(XX[1] > -0.5 * h + box[1, 1])
    I_DIR = np.unique(np.concatenate((I_D, I_U)))
    return np.setdiff1d(I_L, I_DIR), np.setdiff1d(I_R, I_DIR), I_DIR


class FDDisc:
    """Five-point discretisation of -c11 u_xx - c22 u_yy - 2 c12 u_xy + c1 u_x + c u
    on the grid of spacing h (fd_disc.py:83-140)."""

    def __init__(self, box_geom, h, pdo):
        self.box, self.h, self.pdo = np.asarray(box_geom, dtype=float), h, pdo
        XX, self.n0, self.n1 = grid(box_geom, h)
        self.XX = XX.T                                     # (N, 2)
        self.I_L, self.I_R, self.I_DIR = boundary_indices(XX, box_geom, h)
        self.I_X = np.unique(np.concatenate((self.I_L, self.I_R, self.I_DIR)))
        self.I_C = np.setdiff1d(np.arange(self.XX.shape[0]), self.I_X)
        self.ns = np.array([self.n0, self.n1])

    def assemble_sparse(self):
        h, op, n0, n1 = self.h, self.pdo, self.n0, self.n1
        N = n0 * n1
        d0sq = (1 / (h * h)) * sp.diags([1, -2, 1], [-1, 0, 1], shape=(n0, n0), format='csc', dtype=np.float64)
        d1sq = (1 / (h * h)) * sp.diags([1, -2, 1], [-1, 0, 1], shape=(n1, n1), format='csc', dtype=np.float64)
        d0 = (1 / (2 * h)) * sp.diags([-1, 0, +1], [-1, 0, 1], shape=(n0, n0), format='csc', dtype=np.float64)
        d1 = (1 / (2 * h)) * sp.diags([-1, 0, +1], [-1, 0, 1], shape=(n1, n1), format='csc', dtype=np.float64)
        D00 = sp.kron(d0sq, sp.eye(n1))
        D11 = sp.kron(sp.eye(n0), d1sq)
        diag = lambda key: sp.diags(np.asarray(op[key](self.XX), dtype=float).reshape(N), 0, shape=(N, N))
        A = -diag('c11') @ D00 - diag('c22') @ D11
        if op.get('c12') is not None:
            A -= 2 * diag('c12') @ sp.kron(d0, d1)
        if op.get('c1') is not None:
            A += diag('c1') @ sp.kron(d0, sp.eye(n1))
        if op.get('c2') is not None:
            raise ValueError('the reference cannot assemble a c2 term (fd_disc.py:133-138)')
        if op.get('c') is not None:
            A += diag('c')
        return A


class FDPartition:
    """Slab split of the FD grid and the reduced index sets (slablu_solver.py:83-120, 212-296)."""

    def __init__(self, fd, buf_constant=0.6):
        ns = fd.ns
        n = int(ns.max())
        buf = (n - 1) ** (2 / 3) * buf_constant
        buf_prime = np.sqrt(buf)
        buf = nearest_divisor(int(ns[0]) - 1, int(buf) + 1)
        buf_prime = nearest_divisor(int(ns[1]) - 1, int(buf_prime) + 1)
        self.buf, self.buf_prime = buf, buf_prime
        self.Npan = int(ns[0] / buf)
        self.Npan_loc = int(ns[1] / buf_prime)
        W = (buf + 1) * int(ns[1])
        self.inds_pans = np.arange(W)[None, :] + (np.arange(self.Npan) * buf * int(ns[1]))[:, None]
        self.elim_nblocks, self.elim_bs = buf - 1, buf_prime - 1
        self.rem_nblocks, self.rem_bs = self.Npan_loc - 1, buf - 1
        m = int(ns[1]) - 1
        self.I_L = np.arange(1, m)
        self.I_R = np.arange(1, m) + buf * (m + 1)
        self.I_D = np.arange(0, (buf + 1) * m, m + 1)
        self.I_U = np.arange(0, (buf + 1) * m, m + 1) + m
        I_C = np.concatenate([np.arange(m + 1, buf * m + 1, m + 1) + j for j in range(1, m)])
        # columns of the slab grouped into Npan_loc strips (elim) and their separators (rem)
        I_elim = np.zeros((self.Npan_loc, self.elim_nblocks * self.elim_bs), dtype=np.int64)
        I_rem = np.zeros((self.rem_nblocks, self.rem_bs), dtype=np.int64)
        for j in range(m - 1):
            part, rem = j // buf_prime, j % buf_prime
            cols = np.arange(j * (buf - 1), (j + 1) * (buf - 1))
            if rem == buf_prime - 1:
                I_rem[part] = cols
            else:
                I_elim[part, rem * (buf - 1):(rem + 1) * (buf - 1)] = cols
        self.I_C = np.concatenate([np.sort(I_C[I_elim[j]]) for j in range(self.Npan_loc)] +
                                  [np.sort(I_C[I_rem[j]]) for j in range(self.Npan_loc - 1)])
        ip = self.inds_pans
        self.periodic = False
        self.I_slabC = ip[:, self.I_C].ravel()
        self.I_slabX = ip[1:, self.I_L].ravel()
        self.I_Ctot = np.concatenate((self.I_slabC, self.I_slabX))
        I_Ddir = np.concatenate((ip[0, self.I_D], ip[1:, self.I_D[1:]].ravel()))
        I_Udir = np.concatenate((ip[0, self.I_U], ip[1:, self.I_U[1:]].ravel()))
        self.I_Xtot = np.concatenate((ip[0, self.I_L], ip[-1, self.I_R], I_Ddir, I_Udir))


def solve(fd, part, A, u_dir_func):
    """superLU black-box solve on the FD grid (slablu_solver.py:601-666): the grid
    solution with the Dirichlet values, and the reduced system's relative residual."""
    from .domain import solve_superlu
    u_dir = np.asarray(u_dir_func(fd.XX[part.I_Xtot]), dtype=float).reshape(part.I_Xtot.size, -1)
    x, ff, res = solve_superlu(None, part, A.tocsr(), u_dir)
    sol = np.zeros((fd.XX.shape[0], u_dir.shape[1]))
    sol[part.I_Ctot] = x
    sol[part.I_Xtot] = u_dir
    return sol, res
