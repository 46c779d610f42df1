"""Oracle: the full HPS collocation system and its adjoint, dense FP64 (test infrastructure only).

The reference solves the face system built from leaf DtN maps
(src_disc/hps_multidomain_disc.py:84-95) and recovers leaf interiors afterwards
(src_disc/hps_parallel_leaf_ops.py:73-92).  Eliminating nothing, the same
discretisation is one sparse system over [interior nodes of every leaf ; faces
without Dirichlet data]:
  interior PDE rows  Aloc[Jc, :] u_leaf = f          (hps_parallel_leaf_ops.py:17-27)
  face flux rows     sum over the leaves of a face of Nx[s, :] u_leaf = 0
                     (the rows that the DtN maps Nx[:,Jc] S + Nx[:,Jx] condense, :50-58).
With a mixed derivative (c12) the interior PDE rows see the leaf boundary
through Interp_mat, corners included (the c12 branch of form_DtNs, :59-65,
84-92): their face columns are Aloc[Jc, Jxreorder] Interp_mat, while the flux
rows keep Nx on the face values themselves.
This module assembles that system with SciPy, solves it directly, and computes
gradients of L = sum(w * u) at the leaf nodes by the transposed solve: a dense
FP64 reference gradient independent of the GPU engine's factor reuse.
The reference has no adjoint; this is a restatement of the standard one.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import leaf as leafmod

KEYS = ('c11', 'c22', 'c12', 'c1', 'c2', 'c')


class Collocation:
    """K_UU u_U = f_U - K_UD u_D with U = [interior (leaf*n + r) ; non-Dirichlet faces]."""

    def __init__(self, md, part, coeffs):
        ld = md.ld
        self.md, self.part, self.coeffs = md, part, coeffs
        nl, p = md.nboxes, md.p
        n, nx = ld.Jc.size, ld.Jx.size
        self.n, self.nx = n, nx
        fidx = md.face_index()                      # (nl, nx) global face index
        dmask = np.zeros(md.ntot, dtype=bool)
        dmask[part.I_Xtot] = True
        self.dmask = dmask
        self.upos = -np.ones(md.ntot, dtype=np.int64)
        nd = np.flatnonzero(~dmask)
        self.upos[nd] = nl * n + np.arange(nd.size)
        self.dpos = -np.ones(md.ntot, dtype=np.int64)
        self.dpos[part.I_Xtot] = np.arange(part.I_Xtot.size)
        self.nU = nl * n + nd.size
        self.fidx = fidx
        A = leafmod.aloc(ld, coeffs)                # (nl, p^2, p^2)
        self.A = A
        self.mixed = coeffs.get('c12') is not None
        rows_uu, cols_uu, vals_uu, rows_ud, cols_ud, vals_ud = [], [], [], [], [], []
        leaf = np.arange(nl)
        # interior PDE rows
        r_int = leaf[:, None] * n + np.arange(n)[None, :]                    # (nl, n)
        Acc = A[:, ld.Jc][:, :, ld.Jc]
        if self.mixed:   # the interpolated boundary, corners included
            Acx = A[:, ld.Jc][:, :, ld.Jxreorder] @ ld.Interp_mat[None]
        else:
            Acx = A[:, ld.Jc][:, :, ld.Jx]
        rows_uu.append(np.repeat(r_int[:, :, None], n, axis=2).ravel())
        cols_uu.append(np.repeat(r_int[:, None, :], n, axis=1).ravel())
        vals_uu.append(Acc.ravel())
        self._face_cols(np.repeat(r_int[:, :, None], nx, axis=2), np.repeat(fidx[:, None, :], n, axis=1), Acx,
                        rows_uu, cols_uu, vals_uu, rows_ud, cols_ud, vals_ud)
        # face flux rows, summed over the leaves of each face
        row_f = self.upos[fidx]                                               # (nl, nx), -1 on Dirichlet
        keep = row_f >= 0
        Nc = np.broadcast_to(ld.Nx[:, ld.Jc], (nl, nx, n))
        Nxx = np.broadcast_to(ld.Nx[:, ld.Jx], (nl, nx, nx))
        rr = np.repeat(row_f[:, :, None], n, axis=2)
        cc = np.repeat(r_int[:, None, :], nx, axis=1)
        m = np.repeat(keep[:, :, None], n, axis=2)
        rows_uu.append(rr[m]); cols_uu.append(cc[m]); vals_uu.append(Nc[m])
        rr = np.repeat(row_f[:, :, None], nx, axis=2)
        m = np.repeat(keep[:, :, None], nx, axis=2)
        self._face_cols(rr, np.repeat(fidx[:, None, :], nx, axis=1), Nxx, rows_uu, cols_uu, vals_uu, rows_ud,
                        cols_ud, vals_ud, rowmask=m)
        cat = np.concatenate
        self.K_UU = sp.coo_matrix((cat(vals_uu), (cat(rows_uu), cat(cols_uu))), shape=(self.nU, self.nU)).tocsc()
        self.K_UD = sp.coo_matrix((cat(vals_ud), (cat(rows_ud), cat(cols_ud))),
                                  shape=(self.nU, part.I_Xtot.size)).tocsr()
        self._lu = None
        self._luT = None

    def _face_cols(self, rows, gface, vals, ru, cu, vu, rd, cd, vd, rowmask=None):
        m_all = np.ones(rows.shape, dtype=bool) if rowmask is None else rowmask
        isd = self.dmask[gface]
        mu = m_all & ~isd
        md_ = m_all & isd
        ru.append(rows[mu]); cu.append(self.upos[gface[mu]]); vu.append(vals[mu])
        rd.append(rows[md_]); cd.append(self.dpos[gface[md_]]); vd.append(vals[md_])

    def solve(self, u_dir, fbody=None):
        """u_dir: (|I_Xtot|, nrhs) in I_Xtot order; fbody: (npts, nrhs) or None.
        Returns (u_U, u_faces (ntot, nrhs), sol_tot (npts, nrhs))."""
        md, ld = self.md, self.md.ld
        u_dir = np.asarray(u_dir, dtype=float).reshape(self.part.I_Xtot.size, -1)
        nrhs = u_dir.shape[1]
        f = -(self.K_UD @ u_dir)
        if fbody is not None:
            fb = np.asarray(fbody, dtype=float).reshape(md.nboxes, md.p ** 2, nrhs)
            f[: md.nboxes * self.n] += fb[:, ld.Jc].reshape(-1, nrhs)
        if self._lu is None:
            self._lu = spla.splu(self.K_UU)
        uU = self._lu.solve(f).reshape(self.nU, nrhs)
        ufaces = np.zeros((md.ntot, nrhs))
        nd = np.flatnonzero(~self.dmask)
        ufaces[nd] = uU[self.upos[nd]]
        ufaces[self.part.I_Xtot] = u_dir
        return uU, ufaces, self.assemble(uU, ufaces)

    def assemble(self, uU, ufaces):
        """Leaf-node solution: interiors, and Interp_mat on each leaf boundary (form_DtNs 'solve')."""
        md, ld = self.md, self.md.ld
        nrhs = uU.shape[1]
        u = np.zeros((md.nboxes, md.p ** 2, nrhs))
        u[:, ld.Jc] = uU[: md.nboxes * self.n].reshape(md.nboxes, self.n, nrhs)
        u[:, ld.Jxreorder] = ld.Interp_mat[None] @ ufaces[self.fidx]
        return u.reshape(-1, nrhs)

    def leaf_full(self, uU, ufaces):
        """Per-leaf node values with interiors and face nodes set (corners 0)."""
        md, ld = self.md, self.md.ld
        nrhs = uU.shape[1]
        u = np.zeros((md.nboxes, md.p ** 2, nrhs))
        u[:, ld.Jc] = uU[: md.nboxes * self.n].reshape(md.nboxes, self.n, nrhs)
        u[:, ld.Jx] = ufaces[self.fidx]
        return u

    def gradient(self, uU, ufaces, w):
        """Gradients of L = sum(w * sol_tot) (w: (npts, nrhs)).

        Returns dict: 'lam_leaf' (npts, nrhs) multipliers of the interior rows at
        the leaf nodes (= dL/dfbody), 'lam_faces' (ntot, nrhs), 'bnd' (|I_Xtot|,
        nrhs) = dL/du_dir, and dL/d<coefficient> (npts,) summed over rhs for each
        coefficient present."""
        md, ld = self.md, self.md.ld
        nl, p = md.nboxes, md.p
        w = np.asarray(w, dtype=float).reshape(nl, p * p, -1)
        nrhs = w.shape[2]
        g_int = w[:, ld.Jc].reshape(-1, nrhs)
        g_leaf_faces = np.swapaxes(ld.Interp_mat, 0, 1)[None] @ w[:, ld.Jxreorder]   # (nl, nx, nrhs)
        g_faces = np.zeros((md.ntot, nrhs))
        np.add.at(g_faces, self.fidx.ravel(), g_leaf_faces.reshape(-1, nrhs))
        nd = np.flatnonzero(~self.dmask)
        gU = np.zeros((self.nU, nrhs))
        gU[: nl * self.n] = g_int
        gU[self.upos[nd]] = g_faces[nd]
        if self._luT is None:
            self._luT = spla.splu(self.K_UU.T.tocsc())
        lam = self._luT.solve(gU).reshape(self.nU, nrhs)
        out = {}
        out['bnd'] = g_faces[self.part.I_Xtot] - self.K_UD.T @ lam
        lam_c = lam[: nl * self.n].reshape(nl, self.n, nrhs)
        lam_leaf = np.zeros((nl, p * p, nrhs))
        lam_leaf[:, ld.Jc] = lam_c
        out['lam_leaf'] = lam_leaf.reshape(-1, nrhs)
        lam_faces = np.zeros((md.ntot, nrhs))
        lam_faces[nd] = lam[self.upos[nd]]
        out['lam_faces'] = lam_faces
        # the node values the PDE rows see: face values, or with c12 the interpolated boundary
        if self.mixed:
            u = self.assemble(uU, ufaces).reshape(nl, p * p, nrhs)
        else:
            u = self.leaf_full(uU, ufaces)                                         # (nl, p^2, nrhs)
        ops = {'c11': (ld.D11, -1.0), 'c22': (ld.D22, -1.0), 'c12': (ld.D12, -2.0), 'c1': (ld.D1, 1.0),
               'c2': (ld.D2, 1.0)}
        for key in KEYS:
            if self.coeffs.get(key) is None:
                continue
            if key == 'c':
                dAu = u                                                            # d(Au)_k/dc_k = u_k
            else:
                Dm, sgn = ops[key]
                dAu = sgn * np.einsum('kj,ljr->lkr', Dm, u)                        # d(Au)_k/dc11_k = -(D11 u)_k ...
            g = np.zeros((nl, p * p))
            g[:, ld.Jc] = -(lam_c * dAu[:, ld.Jc]).sum(axis=2)
            out[key] = g.reshape(-1)
        return out
