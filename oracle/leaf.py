"""Oracle: leaf spectral discretisation and leaf DtN maps (test infrastructure only).

Restates, in NumPy and FP64,
  src_disc/hps_subdomain_disc.py:16-25    cheb
  src_disc/hps_subdomain_disc.py:30-37    get_loc_interp
  src_disc/hps_subdomain_disc.py:53-80    HPS_Disc._get_interp_mat
  src_disc/hps_subdomain_disc.py:83-100   HPS_Disc.get_diff_ops (2-D branch)
  src_disc/hps_subdomain_disc.py:105-152  leaf_discretization_2d, cheb_2d
  src_disc/hps_parallel_leaf_ops.py:10-37 get_Aloc_2d / Aloc_acc
  src_disc/hps_parallel_leaf_ops.py:40-92 form_DtNs ('build' and 'solve', with and without c12)
"""
from dataclasses import dataclass

import numpy as np
import numpy.polynomial.chebyshev as npcheb


def cheb(m):
    """Chebyshev differentiation matrix on the m+1 points cos(pi k/m).

    Follows src_disc/hps_subdomain_disc.py:16-25: off-diagonal c_i/(c_j (x_i-x_j)),
    then the diagonal is fixed so that every row sums to zero (the row sum is
    taken with a unit placeholder on the diagonal, as the reference does).
    """
    k = np.arange(m + 1)
    x = np.cos(np.pi * k / m)
    c = np.ones(m + 1)
    c[0] = 2.0
    c[-1] = 2.0
    c = c * (-1.0) ** k
    diff = x[:, None] - x[None, :]
    D = (c[:, None] * (1.0 / c)[None, :]) / (diff + np.eye(m + 1))
    D = D - np.diag(D.sum(axis=1))
    return D, x


@dataclass
class LeafDisc:
    p: int
    a: float
    zz: np.ndarray          # (2, p^2) node coordinates relative to the leaf centre
    D: np.ndarray           # (p, p) 1-D derivative on ascending nodes, scaled by 1/a (sign as in the reference)
    D1: np.ndarray          # (p^2, p^2)
    D2: np.ndarray
    D11: np.ndarray
    D22: np.ndarray
    D12: np.ndarray
    Jl: np.ndarray
    Jr: np.ndarray
    Jd: np.ndarray
    Ju: np.ndarray
    Jx: np.ndarray
    Jc: np.ndarray
    Jxreorder: np.ndarray
    Nx: np.ndarray          # (4(p-2), p^2)
    Interp_mat: np.ndarray  # (4(p-1), 4(p-2))
    interp_q: int


def cheb_2d(a, p):
    """Tensor Chebyshev grid and Kronecker operators (hps_subdomain_disc.py:136-152)."""
    D, x = cheb(p - 1)
    xvec = a * x[::-1]
    D = (1 / a) * D
    I = np.eye(p)
    D1 = -np.kron(D, I)
    D2 = -np.kron(I, D)
    Dsq = D @ D
    D11 = np.kron(Dsq, I)
    D22 = np.kron(I, Dsq)
    D12 = np.kron(D, D)
    zz = np.vstack((np.repeat(xvec, p), np.tile(xvec, p)))
    return zz, D, D1, D2, D11, D22, D12


def _interp_fit(x_all, x_inner, q):
    """Least-squares Chebyshev-Vandermonde interpolation (hps_subdomain_disc.py:30-37)."""
    V_all = npcheb.chebvander(x_all, q)
    V_in = npcheb.chebvander(x_inner, q)
    M = np.linalg.lstsq(V_in.T, V_all.T, rcond=None)[0].T
    err = np.linalg.norm(M @ V_in - V_all)
    cond = np.linalg.cond(M)
    return M, err, cond


def interp_mat(zz, a, p):
    """Face-to-(face+corner) interpolation operator (hps_subdomain_disc.py:53-80)."""
    x_all = zz[1, : p - 1] + a
    x_inner = zz[1, 1 : p - 1] + a
    q = p + 5
    while True:
        M, err, cond = _interp_fit(x_all, x_inner, q)
        if cond < 3.25 or (err > 2e-8 and cond < 3.5):
            break
        q += 10
    q2 = p - 2
    B = np.zeros((4 * (p - 1), 4 * q2))
    for f in range(4):
        B[f * (p - 1) : (f + 1) * (p - 1), f * q2 : (f + 1) * q2] = M
    # the four diagonal blocks act on faces ordered [L, U, flip(R), flip(D)]
    # (the counter-clockwise walk of Jxreorder); permute the columns so the
    # operator takes face data in the [L, R, D, U] order of Jx
    order = np.concatenate((np.arange(q2), np.arange(q2) + 3 * q2,
                            np.arange(q2)[::-1] + q2, np.arange(q2)[::-1] + 2 * q2))
    return B[:, np.argsort(order)], q


def leaf_disc(a, p):
    """Index sets and operators of one leaf (hps_subdomain_disc.py:83-134)."""
    zz, D, D1, D2, D11, D22, D12 = cheb_2d(a, p)
    h = zz[1, 1] - zz[0, 1]
    in0 = np.abs(zz[0]) < a - 0.5 * h
    in1 = np.abs(zz[1]) < a - 0.5 * h
    Jl = np.flatnonzero((zz[0] < -a + 0.5 * h) & in1)
    Jr = np.flatnonzero((zz[0] > a - 0.5 * h) & in1)
    Jd = np.flatnonzero((zz[1] < -a + 0.5 * h) & in0)
    Ju = np.flatnonzero((zz[1] > a - 0.5 * h) & in0)
    Jc = np.flatnonzero(in0 & in1)
    Jx = np.concatenate((Jl, Jr, Jd, Ju))
    corners = np.setdiff1d(np.arange(p * p), np.concatenate((Jc, Jx)))
    Jxreorder = np.concatenate(([corners[0]], Jl, [corners[1]], Ju,
                                [corners[3]], Jr[::-1], [corners[2]], Jd[::-1]))
    Nx = np.concatenate((-D1[Jl], D1[Jr], -D2[Jd], D2[Ju]))
    Imat, q = interp_mat(zz, a, p)
    return LeafDisc(p=p, a=a, zz=zz, D=D, D1=D1, D2=D2, D11=D11, D22=D22, D12=D12,
                    Jl=Jl, Jr=Jr, Jd=Jd, Ju=Ju, Jx=Jx, Jc=Jc, Jxreorder=Jxreorder,
                    Nx=Nx, Interp_mat=Imat, interp_q=q)


def aloc(ld, coeffs):
    """Dense leaf operators for a batch of leaves (hps_parallel_leaf_ops.py:10-37).

    ``coeffs`` maps 'c11', 'c22', 'c12', 'c1', 'c2', 'c' to arrays (nleaf, p^2)
    of coefficient values at the leaf nodes (absent keys are zero terms), added
    in the reference's order with its factors (-1, -1, -2, 1, 1).  Returns
    (nleaf, p^2, p^2).
    """
    terms = [('c11', ld.D11, -1.0), ('c22', ld.D22, -1.0), ('c12', ld.D12, -2.0), ('c1', ld.D1, 1.0),
             ('c2', ld.D2, 1.0)]
    nleaf = next(iter(coeffs.values())).shape[0]
    n = ld.p * ld.p
    A = np.zeros((nleaf, n, n))
    for key, Dmat, s in terms:
        if coeffs.get(key) is not None:
            A += (s * coeffs[key])[:, :, None] * Dmat[None]
    if coeffs.get('c') is not None:
        A += coeffs['c'][:, :, None] * np.eye(n)[None]
    return A


def dtn_build(ld, coeffs, return_S=False):
    """Leaf DtN maps (form_DtNs 'build', hps_parallel_leaf_ops.py:50-65).

    S = -A_cc^{-1} A_cx ; DtN = Nx[:, Jc] S + Nx[:, Jx].  With a mixed
    derivative (c12), the interior couples to the corners too: the columns are
    the 4(p-1) nodes Jxreorder and S = -A_cc^{-1} A_c,Jxreorder Interp_mat
    (:59-65).
    """
    A = aloc(ld, coeffs)
    Acc = A[:, ld.Jc][:, :, ld.Jc]
    if coeffs.get('c12') is None:
        S = -np.linalg.solve(Acc, A[:, ld.Jc][:, :, ld.Jx])
    else:
        S = -np.linalg.solve(Acc, A[:, ld.Jc][:, :, ld.Jxreorder]) @ ld.Interp_mat[None]
    DtN = ld.Nx[:, ld.Jc][None] @ S + ld.Nx[:, ld.Jx][None]
    return (DtN, S) if return_S else DtN


def dtn_solve(ld, coeffs, u_face, f_body=None):
    """Leaf interior recovery and local residual (form_DtNs 'solve', :73-92).

    u_face: (nleaf, 4(p-2), nrhs) face values in [L, R, D, U] order.
    Returns (u_leaf (nleaf, p^2, nrhs), residual (nleaf, p^2, nrhs)) where the
    residual is nonzero only at Jc, as in the reference.
    """
    A = aloc(ld, coeffs)
    nleaf, _, nrhs = u_face.shape
    n = ld.p * ld.p
    Acc = A[:, ld.Jc][:, :, ld.Jc]
    fb = np.zeros((nleaf, ld.Jc.size, nrhs)) if f_body is None else f_body
    u = np.zeros((nleaf, n, nrhs))
    u[:, ld.Jxreorder] = ld.Interp_mat[None] @ u_face
    if coeffs.get('c12') is None:
        u[:, ld.Jc] = np.linalg.solve(Acc, fb - A[:, ld.Jc][:, :, ld.Jx] @ u_face)
    else:  # the interior sees the interpolated boundary, corners included (:84-88)
        u[:, ld.Jc] = np.linalg.solve(Acc, fb - A[:, ld.Jc][:, :, ld.Jxreorder] @ u[:, ld.Jxreorder])
    res = np.zeros((nleaf, n, nrhs))
    res[:, ld.Jc] = A[:, ld.Jc] @ u - fb
    return u, res
