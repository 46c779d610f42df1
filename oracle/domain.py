"""Oracle: multidomain HPS assembly, slab partition and FP64 solves (test infrastructure only).

Restates, in NumPy/SciPy and FP64,
  src_disc/hps_multidomain_disc.py:19-51    HPS_Multidomain.__init__ (box count, grid)
  src_disc/hps_multidomain_disc.py:53-109   sparse_mat (face numbering, COO -> CSR)
  src_disc/hps_multidomain_disc.py:111-124  get_grid
  src_disc/hps_multidomain_disc.py:126-182  get_unique_inds
  src_disc/hps_multidomain_disc.py:227-243  solve (leaf recovery)
  src_solver/slablu_solver.py:35-46         get_nearest_div
  src_solver/slablu_solver.py:61-123        Domain_Solver.__init__ (I_Ctot, I_Xtot)
  src_solver/slablu_solver.py:127-202       hps_disc / hps_panel_split
  src_solver/slablu_solver.py:360-385,414-433,601-620  superLU black-box path (the FP64
                                            oracle), with the periodic fold
  src_solver/slablu_solver.py:297-358,543-599,901-943  two-level slab solve
  src_solver/slablu_solver.py:89-120,489-541,1232-1303  periodic partition, right-hand
                                            side and cyclic interface assembly
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import leaf as leafmod
from . import block_tridiag as bt


def nearest_divisor(n, x):
    """Divisor of n closest to x, ties to the larger (slablu_solver.py:35-46)."""
    best, dist = n, abs(n - x)
    for i in range(1, int(n ** 0.5) + 1):
        if n % i:
            continue
        for f in (i, n // i):
            d = abs(f - x)
            if d < dist or (d == dist and f > best):
                best, dist = f, d
    return best


class Multidomain:
    """Leaf grid and reduced face system of the unit-square HPS discretisation."""

    def __init__(self, box_geom, a, p):
        box_geom = np.asarray(box_geom, dtype=float)
        self.p, self.a, self.q = p, a, p - 2
        self.n = np.rint((box_geom[:, 1] - box_geom[:, 0]) / (2 * a)).astype(int)
        self.n0, self.n1 = int(self.n[0]), int(self.n[1])
        self.nboxes = self.n0 * self.n1
        self.box_geom = box_geom
        self.ld = leafmod.leaf_disc(a, p)
        self.xx = self.grid()
        self.I_unique, self.I_copy1, self.I_copy2 = self.unique_inds()
        xx_ext = self.xx[:, self.ld.Jx, :].reshape(-1, 2)
        self.xx_active = xx_ext[self.I_unique]
        self.xx_tot = self.xx.reshape(-1, 2)
        self.ntot = self.q * (self.n0 * (2 * self.n1 + 1) + self.n1)

    def grid(self):
        """Leaf node coordinates, box index i*n1 + j (hps_multidomain_disc.py:111-124)."""
        zz = self.ld.zz.T
        i = np.repeat(np.arange(self.n0), self.n1)
        j = np.tile(np.arange(self.n1), self.n0)
        xx = np.empty((self.nboxes, self.p ** 2, 2))
        xx[:, :, 0] = zz[None, :, 0] + (self.a + 2 * self.a * i + self.box_geom[0, 0])[:, None]
        xx[:, :, 1] = zz[None, :, 1] + (self.a + 2 * self.a * j + self.box_geom[1, 0])[:, None]
        return xx

    def face_index(self):
        """Global reduced index of each leaf's [L, R, D, U] face nodes (hps_multidomain_disc.py:63-81)."""
        q, n1 = self.q, self.n1
        i = np.repeat(np.arange(self.n0), n1)
        j = np.tile(np.arange(n1), self.n0)
        off = (2 * n1 + 1) * i
        faces = np.stack((off + j, off + 2 * n1 + 1 + j, off + n1 + j, off + n1 + j + 1), axis=1)
        return (faces[:, :, None] * q + np.arange(q)[None, None, :]).reshape(self.nboxes, 4 * q)

    def unique_inds(self):
        """Map unique face nodes to positions in the per-leaf face array (:126-182)."""
        q, n0, n1 = self.q, self.n0, self.n1
        box = np.arange(n0 * n1 * 4 * q).reshape(n0, n1, 4 * q)
        uniq, c1, c2 = [box[0, :, :q].ravel()], [], []
        for i in range(n0):
            if i > 0:
                uniq.append(box[i, :, :q].ravel())
                c1.append(box[i, :, :q].ravel())
                c2.append(box[i - 1, :, q:2 * q].ravel())
            uniq.append(box[i, 0, 2 * q:3 * q])
            d_rep = box[i, 1:, 2 * q:3 * q].ravel()
            uniq.append(d_rep)
            c1.append(d_rep)
            c2.append(box[i, : n1 - 1, 3 * q:].ravel())
            uniq.append(box[i, n1 - 1, 3 * q:])
        uniq.append(box[n0 - 1, :, q:2 * q].ravel())
        cat = lambda L: np.concatenate(L) if L else np.zeros(0, dtype=int)
        return cat(uniq), cat(c1), cat(c2)

    def coeffs(self, pdo):
        """Evaluate the PDO coefficient callables at every leaf node (a 'c12' entry
        appears only when the PDO has a mixed derivative)."""
        flat = self.xx.reshape(-1, 2)
        out = {}
        keys = ('c11', 'c22', 'c1', 'c2', 'c') + (('c12',) if pdo.get('c12') is not None else ())
        for key in keys:
            f = pdo.get(key)
            out[key] = None if f is None else np.asarray(f(flat), dtype=float).reshape(self.nboxes, -1)
        return out

    def sparse_mat(self, dtn):
        """Sum leaf DtN maps into the reduced CSR operator (hps_multidomain_disc.py:84-95)."""
        idx = self.face_index()
        m = idx.shape[1]
        rows = np.repeat(idx, m, axis=1).ravel()
        cols = np.tile(idx, (1, m)).ravel()
        return sp.coo_matrix((dtn.ravel(), (rows, cols)), shape=(self.ntot, self.ntot)).tocsr()

    def face_to_leaf(self, u_active):
        """Scatter reduced face values to per-leaf [L, R, D, U] arrays (:232-236)."""
        nrhs = u_active.shape[-1]
        bnd = np.zeros((self.nboxes * 4 * self.q, nrhs))
        bnd[self.I_unique] = u_active
        bnd[self.I_copy2] = bnd[self.I_copy1]
        return bnd.reshape(self.nboxes, 4 * self.q, nrhs)


class SlabPartition:
    """Slab split of the leaf grid (slablu_solver.py:61-123, 127-202)."""

    def __init__(self, md, buf_constant=1.0, periodic=False):
        q, n0, n1 = md.q, md.n0, md.n1
        self.periodic = bool(periodic)
        n_tmp = max(n0, n1) * q - 1
        buf_points = min(400, int(n_tmp ** (2 / 3) * buf_constant))
        buf = max(int(buf_points / q) + 1, 2)
        buf = nearest_divisor(n0, buf)
        self.buf, self.Npan, self.n1, self.q = buf, n0 // buf, n1, q
        nfaces_pan = (2 * n1 + 1) * buf + n1
        self.inds_pans = (np.arange(nfaces_pan * q)[None, :]
                          + ((2 * n1 + 1) * buf * q * np.arange(self.Npan))[:, None])
        self.I_L = np.arange(n1 * q)
        self.I_R = np.arange(n1 * q) + (2 * n1 + 1) * buf * q
        face = lambda f: f * q + np.arange(q)
        self.I_D = np.concatenate([face((2 * n1 + 1) * b + n1) for b in range(buf)])
        self.I_U = np.concatenate([face((2 * n1 + 1) * b + 2 * n1) for b in range(buf)])
        I_elim = [face((2 * n1 + 1) * b + j) for j in range(n1) for b in range(1, buf)]
        I_rem = [face((2 * n1 + 1) * b + n1 + j) for j in range(1, n1) for b in range(buf)]
        cat = lambda L: np.concatenate(L) if L else np.zeros(0, dtype=int)
        self.I_elim, self.I_rem = cat(I_elim), cat(I_rem)
        self.I_C = np.concatenate((self.I_elim, self.I_rem))
        self.elim_m, self.elim_bs = buf - 1, q
        self.rem_m, self.rem_bs = n1 - 1, buf * q
        ip = self.inds_pans
        self.I_slabC = ip[:, self.I_C].ravel()
        if not self.periodic:
            self.I_slabX = ip[1:, self.I_L].ravel()
            self.I_Xtot = np.concatenate((ip[0, self.I_L], ip[-1, self.I_R],
                                          ip[:, self.I_D].ravel(), ip[:, self.I_U].ravel()))
        else:
            # the left edge of slab 0 and the right edge of the last slab are the
            # same curve: both stay in I_Ctot (the right one last), and only the
            # bottom and top faces carry Dirichlet data (slablu_solver.py:89-120)
            self.I_slabX = np.concatenate((ip[:, self.I_L].ravel(), ip[-1, self.I_R]))
            self.I_Xtot = np.concatenate((ip[:, self.I_D].ravel(), ip[:, self.I_U].ravel()))
            nL, off = self.I_L.size, self.I_C.size * self.Npan
            self.I_Ctot_unique = np.arange(off + nL * self.Npan)
            self.I_Ctot_copy1 = np.arange(nL) + off
            self.I_Ctot_copy2 = np.arange(nL) + off + nL * self.Npan
        self.I_Ctot = np.concatenate((self.I_slabC, self.I_slabX))


def dirichlet_rhs(A, part, u_dir, fold=True):
    """ff = -A[I_Ctot, I_Xtot] u_dir (slablu_solver.py:489-526).  With a periodic
    partition and ``fold``, the rows of the right edge are added to those of
    the left edge and dropped (:520-524)."""
    ff = -(A[part.I_Ctot][:, part.I_Xtot] @ u_dir)
    if part.periodic and fold:
        ff[part.I_Ctot_copy1] += ff[part.I_Ctot_copy2]
        ff = ff[part.I_Ctot_unique]
    return ff


def periodic_fold(part):
    """Selection matrix P (|I_Ctot| x |unique|): P[k, k] = 1 for the unique
    unknowns and P[copy2_k, copy1_k] = 1.  P^T A_CC P is the reference's folded
    matrix (slablu_solver.py:418-433): the right-edge rows and columns added
    onto the left edge's; at most two nonzero terms meet in an entry, so the
    sums are exact whatever their order."""
    n_all, n_u = part.I_Ctot.size, part.I_Ctot_unique.size
    rows = np.concatenate((part.I_Ctot_unique, part.I_Ctot_copy2))
    cols = np.concatenate((part.I_Ctot_unique, part.I_Ctot_copy1))
    return sp.csr_matrix((np.ones(rows.size), (rows, cols)), shape=(n_all, n_u))


def reduced_matrix(A, part):
    """A_CC of the reduced system, folded for a periodic partition."""
    A_CC = A[part.I_Ctot][:, part.I_Ctot]
    if part.periodic:
        P = periodic_fold(part)
        A_CC = P.T @ A_CC @ P
    return A_CC.tocsc()


def solve_superlu(md, part, A, u_dir):
    """FP64 sparse direct solve of the reduced system (slablu_solver.py:360-385,
    414-433, 601-620).

    Returns the reduced solution (on I_Ctot; on its unique part for a periodic
    partition), the RHS and ||A_CC x - f|| / ||f||.
    """
    A_CC = reduced_matrix(A, part)
    ff = dirichlet_rhs(A, part, u_dir)
    lu = spla.splu(A_CC)
    x = lu.solve(ff)
    x = x.reshape(ff.shape)
    res = np.linalg.norm(A_CC @ x - ff) / np.linalg.norm(ff)
    return x, ff, res


def assemble_solution(md, part, x, u_dir):
    """sol_tot on all unique face nodes (slablu_solver.py:630-642); for a periodic
    partition x is on the unique unknowns and the right edge takes the left
    edge's values."""
    sol = np.zeros((md.ntot, x.shape[-1]))
    if part.periodic:
        sol[part.I_Ctot[part.I_Ctot_unique]] = x
        sol[part.I_Ctot[part.I_Ctot_copy2]] = x[part.I_Ctot_copy1]
    else:
        sol[part.I_Ctot] = x
    sol[part.I_Xtot] = u_dir
    return sol


def leaf_recover(md, coeffs, sol_faces):
    """Leaf interior recovery + local residual norm (hps_multidomain_disc.py:227-243)."""
    u_face = md.face_to_leaf(sol_faces)
    u, res = leafmod.dtn_solve(md.ld, coeffs, u_face)
    return u.reshape(-1, u.shape[-1]), float(np.linalg.norm(res))


def solve_full(md, part, coeffs, u_dir_func, A=None):
    """Reference black-box path end to end: DtN -> CSR -> splu -> leaf recovery.

    Returns a dict with the leaf-node solution and the reference's diagnostics.
    """
    if A is None:
        A = md.sparse_mat(leafmod.dtn_build(md.ld, coeffs))
    u_dir = np.asarray(u_dir_func(md.xx_active[part.I_Xtot]), dtype=float).reshape(part.I_Xtot.size, -1)
    x, ff, res = solve_superlu(md, part, A, u_dir)
    sol = assemble_solution(md, part, x, u_dir)
    u_tot, resloc = leaf_recover(md, coeffs, sol)
    return dict(A=A, x=x, ff=ff, res=res, sol_faces=sol, sol_tot=u_tot, resloc=resloc)


# ---------------------------------------------------------------------------
# Two-level slab solver with exact dense interface blocks.
# ---------------------------------------------------------------------------

def _blocks_of(Aw, m, bs):
    """Diagonal / sub / super blocks of a block-tridiagonal dense matrix."""
    diag = np.stack([Aw[i * bs:(i + 1) * bs, i * bs:(i + 1) * bs] for i in range(m)])
    sub = np.stack([Aw[(i + 1) * bs:(i + 2) * bs, i * bs:(i + 1) * bs] for i in range(m - 1)]) \
        if m > 1 else np.zeros((0, bs, bs))
    sup = np.stack([Aw[i * bs:(i + 1) * bs, (i + 1) * bs:(i + 2) * bs] for i in range(m - 1)]) \
        if m > 1 else np.zeros((0, bs, bs))
    return diag, sub, sup


class SlabLU:
    """Two-level SlabLU (slablu_solver.py:297-358, 543-599, 668-687, 718-943).

    Level 1 (``Aloc``): per slab row, the vertical interior faces form a
    block-tridiagonal system (m = buf-1 blocks of p-2).  Level 2 (``Ared``):
    per slab, the horizontal interior faces after eliminating level 1 form a
    block-tridiagonal system (m = n1-1 blocks of buf(p-2)).  The slab
    interface operator T = A_XX - A_XC A_CC^{-1} A_CX is formed exactly and
    densely (the reference compresses it with randomised HBS sketches of the
    same operator, src_solver/slablu_solver.py:1139-1308) and the interface
    block-tridiagonal system is factored by the sequential block LU of
    src_solver/block_tridiag_solver_structured.py:34-76.
    """

    def __init__(self, md, part, A):
        self.md, self.part, self.A = md, part, A.tocsr()
        pt = part
        ip = pt.inds_pans
        self.n_elim = pt.I_elim.size
        # Level 1: one block tridiagonal per (slab, row)
        diag, sub, sup = [], [], []
        for s in range(pt.Npan):
            I = ip[s, pt.I_elim]
            Aee = self.A[I][:, I].toarray()
            blk = pt.elim_m * pt.elim_bs
            for r in range(pt.n1):
                d, l, u = _blocks_of(Aee[r * blk:(r + 1) * blk, r * blk:(r + 1) * blk],
                                     pt.elim_m, pt.elim_bs)
                diag.append(d); sub.append(l); sup.append(u)
        self.Aloc = bt.BlockTridiag(np.stack(diag), np.stack(sub), np.stack(sup))
        # Level 2: Ared = A_rr - A_re Aloc^{-1} A_er per slab
        diag, sub, sup = [], [], []
        for s in range(pt.Npan):
            Ie, Ir = ip[s, pt.I_elim], ip[s, pt.I_rem]
            Are = self.A[Ir][:, Ie].toarray()
            Aer = self.A[Ie][:, Ir].toarray()
            Arr = self.A[Ir][:, Ir].toarray()
            Z = self._aloc_solve(s, Aer)
            Ared = Arr - Are @ Z
            d, l, u = _blocks_of(Ared, pt.rem_m, pt.rem_bs)
            diag.append(d); sub.append(l); sup.append(u)
        self.Ared = bt.BlockTridiag(np.stack(diag), np.stack(sub), np.stack(sup))
        # Slab interface operators T_s = A_XX - A_XC A_CC^{-1} A_CX, X = [L; R]
        self.T = []
        for s in range(pt.Npan):
            Ic = ip[s, pt.I_C]
            IX = np.concatenate((ip[s, pt.I_L], ip[s, pt.I_R]))
            Acx = self.A[Ic][:, IX].toarray()
            Axc = self.A[IX][:, Ic].toarray()
            if s < pt.Npan - 1:
                # only A_LL of the diagonal: the R block is counted by the next slab
                nL = pt.I_L.size
                Axx = np.zeros((2 * nL, 2 * nL))
                IL = ip[s, pt.I_L]
                Axx[:nL, :nL] = self.A[IL][:, IL].toarray()
            else:
                Axx = self.A[IX][:, IX].toarray()
            self.T.append(Axx - Axc @ self.slab_solve(s, Acx))
        nL = pt.I_L.size
        Tb = np.stack(self.T)
        if not pt.periodic:
            diagI = Tb[:-1, nL:, nL:] + Tb[1:, :nL, :nL]
            subI = Tb[1:-1, nL:, :nL]
            supI = Tb[1:-1, :nL, nL:]
            self.iface = bt.InterfaceBlockLU(diagI, subI, supI)
        else:
            # interface j is the left edge of slab j, and the right edge of slab
            # j-1 (of the last slab for j = 0): diag_j = T_RR(j-1) + T_LL(j),
            # sub_j = T_RL(j-1), sup_j = T_LR(j) (slablu_solver.py:1260-1303)
            prev = np.roll(np.arange(pt.Npan), 1)
            diagI = Tb[prev, nL:, nL:] + Tb[:, :nL, :nL]
            subI = Tb[prev, nL:, :nL]
            supI = Tb[:, :nL, nL:]
            self.iface = bt.CyclicInterfaceBlockLU(diagI, subI, supI)

    def _aloc_solve(self, s, rhs, transpose=False):
        pt = self.part
        nrow = pt.n1
        blk = pt.elim_m * pt.elim_bs
        f = rhs.reshape(nrow, blk, -1).copy()
        out = self.Aloc.solve(f, b_start=s * nrow, b_end=(s + 1) * nrow, transpose=transpose)
        return out.reshape(nrow * blk, -1)

    def slab_solve(self, s, f, transpose=False):
        """A_CC(slab s)^{-1} f via the two levels (solve_slab, slablu_solver.py:901-943)."""
        pt, ip = self.part, self.part.inds_pans
        Ie, Ir = ip[s, pt.I_elim], ip[s, pt.I_rem]
        ne = Ie.size
        fe, fr = f[:ne], f[ne:]
        y = self._aloc_solve(s, fe, transpose)
        if not transpose:
            fr = fr - self.A[Ir][:, Ie] @ y
        else:
            fr = fr - self.A[Ie][:, Ir].T @ y
        ur = self.Ared.solve(fr.reshape(1, fr.shape[0], -1), b_start=s, b_end=s + 1,
                             transpose=transpose)[0]
        if not transpose:
            fe2 = fe - self.A[Ie][:, Ir] @ ur
        else:
            fe2 = fe - self.A[Ir][:, Ie].T @ ur
        ue = self._aloc_solve(s, fe2, transpose)
        return np.concatenate((ue, ur))

    def solve(self, ff):
        """Reduced solve on I_Ctot ordering (solve_helper, slablu_solver.py:543-599).

        For a periodic partition ff is the unfolded right-hand side on all of
        I_Ctot (get_rhs with sum_body_load=False); the interface right-hand
        side is folded, the cyclic system solved and the left-edge values
        copied to the right edge; the result is on the unique unknowns."""
        pt = self.part
        nC, nL = pt.I_C.size, pt.I_L.size
        nrhs = ff.shape[-1]
        fC = ff[: pt.Npan * nC]
        yC = np.concatenate([self.slab_solve(s, fC[s * nC:(s + 1) * nC]) for s in range(pt.Npan)])
        fX = ff[pt.Npan * nC:] - self.A[pt.I_slabX][:, pt.I_slabC] @ yC
        if pt.periodic:
            fX[:nL] += fX[pt.Npan * nL:]
            fX = fX[:pt.Npan * nL]
            uX = self.iface.solve(fX.reshape(pt.Npan, -1, nrhs)).reshape(-1, nrhs)
            uX = np.concatenate((uX, uX[:nL]))
        else:
            uX = self.iface.solve(fX.reshape(pt.Npan - 1, -1, nrhs)).reshape(-1, nrhs)
        g = fC - self.A[pt.I_slabC][:, pt.I_slabX] @ uX
        uC = np.concatenate([self.slab_solve(s, g[s * nC:(s + 1) * nC]) for s in range(pt.Npan)])
        sol = np.concatenate((uC, uX))
        return sol[pt.I_Ctot_unique] if pt.periodic else sol


def slablu_pipeline(md, part, co, u_dir_func):
    """Reference CPU slabLU end to end, timed like the reference driver
    (argparse_driver.py:169-170, 250-258): leaf DtNs + assembly, two-level slab
    build, solve with leaf recovery.  Returns (leaf-node solution, timings dict)."""
    import time
    t0 = time.perf_counter()
    A = md.sparse_mat(leafmod.dtn_build(md.ld, co))
    t1 = time.perf_counter()
    S = SlabLU(md, part, A)
    t2 = time.perf_counter()
    u_dir = np.asarray(u_dir_func(md.xx_active[part.I_Xtot]), dtype=float).reshape(-1, 1)
    ff = dirichlet_rhs(A, part, u_dir, fold=False)
    x = S.solve(ff)
    sol = assemble_solution(md, part, x, u_dir)
    u_tot, _ = leaf_recover(md, co, sol)
    t3 = time.perf_counter()
    return u_tot, dict(assembly=t1 - t0, build=t2 - t1, solve=t3 - t2, total=t3 - t0)
