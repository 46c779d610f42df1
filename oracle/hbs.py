"""Oracle: HBS (hierarchically block separable) compression from sketches (test infrastructure only).

Restates, in NumPy/SciPy and FP64, src_solver/hbs_reconstruction.py:
  :27-30    get_nearest_div (block size: smallest divisor of n at or above 2k)
  :49-64    HBS_matrix.__init__ (block size, leaf count padded to a power of two)
  :70-94    reconstruct
  :119-132  todense (through the product with the identity)
  :134-148  matvec (with transpose)
  :150-167  calc_inverse / apply_inverse
  :171-233  _calc_Dhat, _add_Dhat, _calc_inverse
  :238-303  _matvec (upward pass, root, downward pass, leaf level)
  :355-414  _correct_reconstruction, _store_tensors
  :417-421  pinv_right (B pinv(A) by least squares)
  :423-496  _reconstruct, calc_null_rowspace, get_decomp_blocks, project_samples
The reference compresses each slab's interface blocks T_LL, T_LR, T_RL, T_RR
(src_solver/slablu_solver.py:1139-1211) from products with random sketches
Omega, Psi (Y = T Omega, Z = T^T Psi); here the sketches are inputs, so a
fixture made with the reference's random draws can be replayed.

Storage (as the reference): with m = 2^L leaf blocks of size bs, the nodes of
level l (0 = leaves) occupy slots [2^(L+1) - 2^(L+1-l), +2^(L-l)) of
UV (b, 2^(L+1)-2, bs, 2k) ([..., :k] = U, [..., k:] = V; 2k x k blocks above the
leaves) and D (b, 2^(L+1)-1, bs, bs) (2k x 2k above the leaves, the root last).
"""
import numpy as np
import scipy.linalg as sla


def nearest_div_up(n, bs):
    """Smallest divisor of n that is >= bs (n itself if none below it), :27-30."""
    while n % bs > 0 and bs < n:
        bs += 1
    return bs


def _T(a):
    return np.swapaxes(a, -1, -2)


def pinv_right(B, A):
    """B pinv(A) as the least-squares solution of A^T X^T = B^T (:417-421; torch's CPU
    lstsq driver is LAPACK gelsy)."""
    At, Bt = _T(A), _T(B)
    shape = np.broadcast_shapes(At.shape[:-2], Bt.shape[:-2])
    At = np.broadcast_to(At, shape + At.shape[-2:])
    Bt = np.broadcast_to(Bt, shape + Bt.shape[-2:])
    out = np.empty(shape + (At.shape[-1], Bt.shape[-1]))
    for idx in np.ndindex(*shape):
        out[idx] = sla.lstsq(At[idx], Bt[idx], lapack_driver='gelsy', check_finite=False)[0]
    return _T(out)


def _qr_reduced(A):
    return np.linalg.qr(A, mode='reduced')[0]


def calc_null_rowspace(A, k):
    """Orthonormal basis of the k-dimensional null space of the rows of A (:423-428):
    the trailing k columns of the complete QR of A^T."""
    m = A.shape[-1] - k
    Q = np.linalg.qr(_T(A), mode='complete')[0]
    return Q[..., m:]


def get_decomp_blocks(Om, Ps, Y, Z, k):
    """Column and row bases and diagonal blocks of one level (:430-455)."""
    P_null = calc_null_rowspace(Om, k)
    Q_null = calc_null_rowspace(Ps, k)
    U = _qr_reduced(Y @ P_null)[..., :k]
    V = _qr_reduced(Z @ Q_null)[..., :k]
    tmp_row = pinv_right(Y, Om)
    tmp_col = pinv_right(Z, Ps)
    D = tmp_row - U @ (_T(U) @ tmp_row)
    tmp = tmp_col - V @ (_T(V) @ tmp_col)
    D = D + U @ (_T(U) @ _T(tmp))
    return U, V, D


def project_samples(Om, Ps, Y, Z, U, V, D):
    """Sketches of the next level up (:457-464)."""
    return (_T(V) @ Om, _T(U) @ (Y - D @ Om), _T(U) @ Ps, _T(V) @ (Z - _T(D) @ Ps))


def _reconstruct(Om, Ps, Y, Z, b, m, bs, k):
    """Level-by-level bases and diagonal blocks, then the root block (:471-496)."""
    decomp_list, m_curr, decomp = [], m, None
    while m_curr > 0:
        if m_curr == m:
            Omb = Om.reshape(Om.shape[0], m, bs, bs + k)
            Psb = Ps.reshape(Ps.shape[0], m, bs, bs + k)
            Yb = Y.reshape(b, m, bs, bs + k)
            Zb = Z.reshape(b, m, bs, bs + k)
        else:
            Omp, Yp, Psp, Zp = project_samples(Omb, Psb, Yb, Zb, *decomp)
            Omb = Omp[..., :3 * k].reshape(b, m_curr, 2 * k, 3 * k)
            Yb = Yp[..., :3 * k].reshape(b, m_curr, 2 * k, 3 * k)
            Psb = Psp[..., :3 * k].reshape(b, m_curr, 2 * k, 3 * k)
            Zb = Zp[..., :3 * k].reshape(b, m_curr, 2 * k, 3 * k)
        if m_curr == 1:
            ns = Omb.shape[-1]
            D_root = pinv_right(Yb.reshape(b, 2 * k, ns), Omb.reshape(b, 2 * k, ns))
            break
        decomp = get_decomp_blocks(Omb, Psb, Yb, Zb, k)
        m_curr = m_curr // 2 if m_curr % 2 == 0 else m_curr // 2 + 1
        decomp_list.append(decomp)
    return decomp_list, D_root


def _correct_reconstruction(b, k, decomp_list, D_root):
    """Move the diagonal k x k blocks of each parent's D into its children's D
    through the children's bases (:355-389)."""
    L = len(decomp_list)
    D_root = D_root.copy()
    decomp_list = [(U, V, D.copy()) for (U, V, D) in decomp_list]
    U, V, D = decomp_list[L - 1]
    tmp = np.zeros((b, 2, k, k))
    tmp[:, 0] = D_root[:, :k, :k]
    D_root[:, :k, :k] = 0.0
    tmp[:, 1] = D_root[:, k:, k:]
    D_root[:, k:, k:] = 0.0
    D += U @ (tmp @ _T(V))
    for l in range(L - 1, 0, -1):
        U, V, D = decomp_list[l]
        nb = D.shape[1]
        tmp = np.zeros((b, 2 * nb, k, k))
        tmp[:, 0::2] = D[:, :, :k, :k]
        D[:, :, :k, :k] = 0.0
        tmp[:, 1::2] = D[:, :, k:, k:]
        D[:, :, k:, k:] = 0.0
        U, V, D = decomp_list[l - 1]
        D += U @ (tmp @ _T(V))
    return decomp_list, D_root


def _level(L, l):
    start = 2 ** (L + 1) - 2 ** (L + 1 - l)
    return start, start + 2 ** (L - l)


def _store_tensors(b, bs, k, decomp_list, D_root):
    L = len(decomp_list)
    nb = 2 ** (L + 1) - 2
    UV = np.zeros((b, nb, bs, 2 * k))
    Dt = np.zeros((b, nb + 1, bs, bs))
    for l, (U, V, D) in enumerate(decomp_list):
        s, e = _level(L, l)
        r = bs if l == 0 else 2 * k
        UV[:, s:e, :r, :k] = U
        UV[:, s:e, :r, k:] = V
        Dt[:, s:e, :r, :r] = D
    Dt[:, -1, :2 * k, :2 * k] = D_root
    return UV, Dt


def _matvec(UV, Dt, L, b, m, bs, k, q, transpose=False):
    """Product with the compressed matrix (or its transpose), :238-303."""
    nr = q.shape[-1]
    qb = q.reshape(q.shape[0], m, bs, nr)
    qhat = np.zeros((b, 2 ** (L + 1) - 2, k, nr))
    sel_up = slice(k, None) if not transpose else slice(None, k)
    sel_dn = slice(None, k) if not transpose else slice(k, None)
    q_hat = _T(UV[:, :m, :, sel_up]) @ qb
    m_curr = m
    qhat[:, :m] = q_hat
    for l in range(1, L):
        qr_ = q_hat.reshape(b, m_curr // 2, 2 * k, nr)
        s, e = _level(L, l)
        q_hat = _T(UV[:, s:e, :2 * k, sel_up]) @ qr_
        m_curr //= 2
        qhat[:, s:e] = q_hat
    root = Dt[:, -1, :2 * k, :2 * k]
    u_hat = (root if not transpose else _T(root)) @ q_hat.reshape(b, m_curr * k, nr)
    u_hat = u_hat.reshape(b, m_curr, k, nr)
    for l in range(L - 1, 0, -1):
        s0, e0 = _level(L, l - 1)
        qh = qhat[:, s0:e0].reshape(b, m_curr, 2 * k, nr)
        s, e = _level(L, l)
        Dl = Dt[:, s:e, :2 * k, :2 * k]
        u_hat = UV[:, s:e, :2 * k, sel_dn] @ u_hat + (Dl if not transpose else _T(Dl)) @ qh
        u_hat = u_hat.reshape(b, m_curr * 2, k, nr)
        m_curr *= 2
    Dleaf = Dt[:, :m]
    if not transpose:
        ub = Dleaf @ qb + UV[:, :m, :, :k] @ u_hat
    else:
        ub = UV[:, :m, :, k:] @ u_hat + _T(Dleaf) @ qb
    return ub.reshape(b, m * bs, nr)


def _calc_inverse(L, k, UV, Dt):
    """Compressed inverse with the same tree layout (:184-233)."""
    Dt = Dt.copy()
    EF = np.zeros_like(UV)
    G = np.zeros_like(Dt)
    Dhat = None
    for l in range(L):
        s, e = _level(L, l)
        r = UV.shape[2] if l == 0 else 2 * k
        U = UV[:, s:e, :r, :k]
        V = UV[:, s:e, :r, k:]
        D = Dt[:, s:e, :r, :r]
        if l > 0:
            for j in range(D.shape[1]):
                D[:, j, :k, :k] += Dhat[:, 2 * j]
                D[:, j, k:, k:] += Dhat[:, 2 * j + 1]
        Dinv = np.linalg.inv(D)
        Dhat = np.linalg.inv(_T(V) @ (Dinv @ U))
        U_solve = Dinv @ U
        V_solve = _T(V) @ Dinv
        E = U_solve @ Dhat
        F = _T(Dhat @ V_solve)
        EF[:, s:e, :r, :k] = E
        EF[:, s:e, :r, k:] = F
        G[:, s:e, :r, :r] = Dinv - U_solve @ _T(F)
    Droot = Dt[:, -1, :2 * k, :2 * k]
    for j in range(Droot.shape[0]):
        Droot[j] += sla.block_diag(*Dhat[j])
    G[:, -1, :2 * k, :2 * k] = np.linalg.inv(Droot)
    return EF, G


class HBSMatrix:
    """Batch of b HBS matrices of size n with rank k (HBS_matrix, :49-167)."""

    def __init__(self, b, n, k, n_pad=0):
        self.b, self.n, self.k = b, n, k
        self.bs = nearest_div_up(n + n_pad, 2 * k)
        self.m = (n + n_pad) // self.bs
        self.n_pad = n_pad
        p = np.log2(self.m)
        if abs(int(p) - p) > 1e-14:
            p = int(p) + 1
            self.n_pad += (2 ** p - self.m) * self.bs
            self.m = 2 ** p

    def reconstruct(self, Omega, Psi, Y, Z, Omega_pad=None, Psi_pad=None):
        """Omega, Psi: (1 or b, n, bs+k) sketches; Y = A Omega, Z = A^T Psi (b, n, bs+k).
        With padding, the reference draws the extra sketch rows at random: pass them
        as Omega_pad, Psi_pad (1 or b, n_pad, bs+k)."""
        b, bs, k = self.b, self.bs, self.k
        if self.n_pad > 0:
            if Omega_pad is None or Psi_pad is None:
                raise ValueError('padded HBS needs the padding sketches')
            Omega = np.concatenate((Omega, Omega_pad), axis=1)
            Psi = np.concatenate((Psi, Psi_pad), axis=1)
            Y = np.concatenate((Y, np.broadcast_to(Omega_pad, (b,) + Omega_pad.shape[1:])), axis=1)
            Z = np.concatenate((Z, np.broadcast_to(Psi_pad, (b,) + Psi_pad.shape[1:])), axis=1)
        decomp, D_root = _reconstruct(Omega, Psi, Y, Z, b, self.m, bs, k)
        decomp, D_root = _correct_reconstruction(b, k, decomp, D_root)
        self.L = len(decomp)
        self.UV, self.D = _store_tensors(b, bs, k, decomp, D_root)
        return self

    def _pad(self, q):
        if self.n_pad == 0:
            return q
        return np.concatenate((q, np.zeros((q.shape[0], self.n_pad, q.shape[2]))), axis=1)

    def matvec(self, q, transpose=False):
        """q: (b, n, nrhs) -> (b, n, nrhs)."""
        out = _matvec(self.UV, self.D, self.L, self.b, self.m, self.bs, self.k, self._pad(q), transpose)
        return out[:, :self.n]

    def todense(self):
        out = np.zeros((self.b, self.n, self.n))
        eye = np.eye(self.n + self.n_pad, self.n)[None]
        for j in range(self.b):
            out[j] = _matvec(self.UV[j:j + 1], self.D[j:j + 1], self.L, 1, self.m, self.bs, self.k, eye)[0, :self.n]
        return out

    def calc_inverse(self):
        self.EF, self.G = _calc_inverse(self.L, self.k, self.UV, self.D)
        return self

    def apply_inverse(self, f, transpose=False):
        out = _matvec(self.EF, self.G, self.L, self.b, self.m, self.bs, self.k, self._pad(f), transpose)
        return out[:, :self.n]
