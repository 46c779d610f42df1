"""Host-side HPS discretisation data for the unit-square leaf grid.

Constant operators of one leaf (Chebyshev differentiation, index sets, normal
derivative rows, face-to-corner interpolation) and the multidomain geometry
(leaf node coordinates, reduced face numbering, slab partition).  Conventions
follow the reference discretisation:
  src_disc/hps_subdomain_disc.py:16-25, 53-80, 83-152   (leaf)
  src_disc/hps_multidomain_disc.py:19-51, 63-81, 111-124 (multidomain)
  src_solver/slablu_solver.py:35-46, 61-202              (slab partition)
Index sets are written in closed form (node k = i1*p + i2, i1 the x index).
"""
import numpy as np
import numpy.polynomial.chebyshev as npcheb


def cheb_matrix(m):
    """Chebyshev points cos(pi k/m) and their differentiation matrix.

    Off-diagonal entries c_i / (c_j (x_i - x_j)); the diagonal makes every row
    sum to zero, computed as in the reference (row sum taken with a unit
    placeholder on the diagonal).
    """
    k = np.arange(m + 1)
    x = np.cos(np.pi * k / m)
    w = np.where((k == 0) | (k == m), 2.0, 1.0) * np.where(k % 2 == 0, 1.0, -1.0)
    dx = x[:, None] - x[None, :] + np.eye(m + 1)
    Dm = np.outer(w, 1.0 / w) / dx
    return Dm - np.diag(Dm.sum(axis=1)), x


class LeafOps:
    """Operators shared by every leaf of half-width ``a`` and order ``p``."""

    def __init__(self, a, p):
        self.a, self.p, self.q = float(a), int(p), int(p) - 2
        p, q = self.p, self.q
        Dm, x = cheb_matrix(p - 1)
        self.xvec = self.a * x[::-1]
        self.D = (1 / self.a) * Dm          # D1 = -kron(D, I), D2 = -kron(I, D)
        self.Dsq = self.D @ self.D
        self.zz = np.vstack((np.repeat(self.xvec, p), np.tile(self.xvec, p)))
        t = np.arange(1, p - 1)
        self.Jl = t.copy()
        self.Jr = (p - 1) * p + t
        self.Jd = t * p
        self.Ju = t * p + p - 1
        self.Jx = np.concatenate((self.Jl, self.Jr, self.Jd, self.Ju))
        self.Jc = (t[:, None] * p + t[None, :]).ravel()
        self.Jxreorder = np.concatenate(([0], self.Jl, [p - 1], self.Ju, [p * p - 1], self.Jr[::-1],
                                         [(p - 1) * p], self.Jd[::-1]))
        self.Nx = self._normal_rows()
        self.Interp_mat, self.interp_q = self._interp()

    def _normal_rows(self):
        """Outward normal-derivative rows at face nodes: [-D1[Jl]; D1[Jr]; -D2[Jd]; D2[Ju]]."""
        p, q, D = self.p, self.q, self.D
        Nx = np.zeros((4 * q, p * p))
        j = np.arange(p)
        for s in range(q):
            i = s + 1
            Nx[s, j * p + i] = D[0, :]                     # -D1 row of node (0, i)
            Nx[q + s, j * p + i] = -D[p - 1, :]            # +D1 row of node (p-1, i)
            Nx[2 * q + s, i * p + j] = D[0, :]             # -D2 row of node (i, 0)
            Nx[3 * q + s, i * p + j] = -D[p - 1, :]        # +D2 row of node (i, p-1)
        return Nx

    def _interp(self):
        """Least-squares Chebyshev interpolation from p-2 face nodes to the
        face plus one corner, block-diagonal over the four faces in the
        counter-clockwise order of Jxreorder, columns in Jx order."""
        p, q = self.p, self.q
        y = self.zz[1]
        xs_all, xs_in = y[: p - 1] + self.a, y[1 : p - 1] + self.a
        deg = p + 5
        while True:
            V_all = npcheb.chebvander(xs_all, deg)
            V_in = npcheb.chebvander(xs_in, deg)
            M = np.linalg.lstsq(V_in.T, V_all.T, rcond=None)[0].T
            err = np.linalg.norm(M @ V_in - V_all)
            cond = np.linalg.cond(M)
            if cond < 3.25 or (err > 2e-8 and cond < 3.5):
                break
            deg += 10
        B = np.kron(np.eye(4), M)
        walk = np.concatenate((np.arange(q), 3 * q + np.arange(q), q + np.arange(q)[::-1],
                               2 * q + np.arange(q)[::-1]))
        inv = np.empty_like(walk)
        inv[walk] = np.arange(4 * q)
        return B[:, inv], deg


def nearest_divisor(n, x):
    """Divisor of n nearest to x; ties go to the larger divisor."""
    divs = [d for d in range(1, n + 1) if n % d == 0]
    return min(divs, key=lambda d: (abs(d - x), -d))


class Geometry:
    """Leaf grid, reduced face numbering and slab partition of a rectangle."""

    def __init__(self, box_geom, a, p, buf_constant=1.0):
        box = np.asarray(box_geom, dtype=float)
        self.box = box
        self.ops = LeafOps(a, p)
        self.a, self.p, self.q = float(a), int(p), int(p) - 2
        self.n = np.rint((box[:, 1] - box[:, 0]) / (2 * a)).astype(int)
        self.n0, self.n1 = int(self.n[0]), int(self.n[1])
        self.nboxes = self.n0 * self.n1
        q, n0, n1 = self.q, self.n0, self.n1
        self.ntot = q * (n0 * (2 * n1 + 1) + n1)
        # leaf node coordinates, leaf index I*n1 + J
        I = np.repeat(np.arange(n0), n1)
        J = np.tile(np.arange(n1), n0)
        zz = self.ops.zz.T
        self.xx = np.empty((self.nboxes, p * p, 2))
        self.xx[:, :, 0] = zz[None, :, 0] + (a + 2 * a * I + box[0, 0])[:, None]
        self.xx[:, :, 1] = zz[None, :, 1] + (a + 2 * a * J + box[1, 0])[:, None]
        self.xx_tot = self.xx.reshape(-1, 2)
        # reduced face numbering of every leaf's [L, R, D, U] nodes
        base = (2 * n1 + 1) * I
        faces = np.stack((base + J, base + 2 * n1 + 1 + J, base + n1 + J, base + n1 + J + 1), axis=1)
        self.leaf_faces = faces
        self.leafglob = (faces[:, :, None] * q + np.arange(q)).reshape(self.nboxes, 4 * q)
        self.xx_active = np.empty((self.ntot, 2))
        self.xx_active[self.leafglob.ravel()] = self.xx[:, self.ops.Jx, :].reshape(-1, 2)
        self._partition(buf_constant)

    def _partition(self, buf_constant):
        q, n0, n1 = self.q, self.n0, self.n1
        n_tmp = max(n0, n1) * q - 1
        buf_points = min(400, int(n_tmp ** (2 / 3) * buf_constant))
        buf = max(int(buf_points / q) + 1, 2)
        self.buf = nearest_divisor(n0, buf)
        self.Npan = n0 // self.buf
        buf, npan = self.buf, self.Npan
        W = (2 * n1 + 1) * buf
        nodes = lambda f: (np.asarray(f)[..., None] * q + np.arange(q)).ravel()
        self.inds_pans = np.arange(W * q + n1 * q)[None, :] + (np.arange(npan) * W * q)[:, None]
        self.I_L = nodes(np.arange(n1))
        self.I_R = nodes(W + np.arange(n1))
        b = np.arange(buf)
        self.I_D = nodes((2 * n1 + 1) * b + n1)
        self.I_U = nodes((2 * n1 + 1) * b + 2 * n1)
        jj, bb = np.meshgrid(np.arange(n1), np.arange(1, buf), indexing='ij')
        I_elim = nodes((2 * n1 + 1) * bb + jj)
        jj, bb = np.meshgrid(np.arange(1, n1), np.arange(buf), indexing='ij')
        I_rem = nodes((2 * n1 + 1) * bb + n1 + jj)
        self.I_C = np.concatenate((I_elim, I_rem))
        ip = self.inds_pans
        self.I_slabC = ip[:, self.I_C].ravel()
        self.I_slabX = ip[1:, self.I_L].ravel()
        self.I_Ctot = np.concatenate((self.I_slabC, self.I_slabX))
        self.I_Xtot = np.concatenate((ip[0, self.I_L], ip[-1, self.I_R], ip[:, self.I_D].ravel(),
                                      ip[:, self.I_U].ravel()))

    @property
    def N_reported(self):
        """Unknown count reported by the reference driver (argparse_driver.py:163)."""
        return self.q * (self.p * self.n0 * self.n1 + self.n0 + self.n1)
