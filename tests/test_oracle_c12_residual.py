"""The FP64 residual with a mixed derivative, as the GPU refinement forms it,
vanishes at the reference's solution (CPU).

With c12 the leaves couple to their corners through Interp_mat.  The engine's
residual (residual_mixed_kernel) evaluates the PDE rows on the interpolated
boundary u[Jxreorder] = Interp_mat u_faces and the flux rows on the face values
themselves.  This restates that split in NumPy and checks it against the
oracle's sparse direct solution of the reference's curvy-annulus discretisation (the
reference's own c12 branch, src_disc/hps_parallel_leaf_ops.py:59-65, 84-92):
if the split differed from the reference's discretisation, the refinement would
converge to a different solution.
"""
import numpy as np

from oracle import domain, funcs
from oracle import leaf as oleaf


def test_mixed_residual_split_vanishes_at_the_reference_solution():
    p, n, kh = 8, 48, 12.0
    a = 1 / (2 * (n / (p - 2)))
    md = domain.Multidomain([[0, 1], [0, 1]], a, p)
    part = domain.SlabPartition(md, 1.0)
    pdo, pmap = funcs.curvy_annulus_pdo(kh, funcs.bfield_constant)
    co = md.coeffs(pdo)
    ud = lambda x: funcs.uu_dir_greens(pmap(x), kh)
    out = domain.solve_full(md, part, co, ud)
    ld = md.ld
    A = oleaf.aloc(ld, co)                                  # (nleaf, p^2, p^2) with the c12 term
    uf = out['sol_faces'][md.face_index()][..., 0]          # (nleaf, 4(p-2)) face values per leaf
    uleaf = out['sol_tot'].reshape(md.nboxes, p * p)
    # PDE rows on the interpolated boundary (corners included)
    u = np.zeros((md.nboxes, p * p))
    u[:, ld.Jc] = uleaf[:, ld.Jc]
    u[:, ld.Jxreorder] = uf @ ld.Interp_mat.T
    r_pde = np.einsum('lij,lj->li', A[:, ld.Jc], u)
    assert np.abs(r_pde).max() < 1e-9 * np.abs(np.einsum('lij,lj->li', np.abs(A[:, ld.Jc]), np.abs(u))).max()
    # without the corners (the c12 term couples every interior node to them) the rows
    # do not vanish; on the raw face values instead of the interpolated ones they do
    # to within the fit's deviation of its face rows from the identity
    corners = np.setdiff1d(np.arange(p * p), np.concatenate((ld.Jc, ld.Jx)))
    u_nc = u.copy()
    u_nc[:, corners] = 0.0
    assert np.abs(np.einsum('lij,lj->li', A[:, ld.Jc], u_nc)).max() > 1e6 * np.abs(r_pde).max()
    u_raw = u.copy()
    u_raw[:, ld.Jx] = uf
    # flux rows on the face values themselves; Nx has no corner columns
    assert np.abs(ld.Nx[:, corners]).max() == 0.0
    flux = u_raw @ ld.Nx.T                                  # (nleaf, 4(p-2))
    rx = np.zeros(md.ntot)
    np.add.at(rx, md.face_index().ravel(), flux.ravel())
    rx[part.I_Xtot] = 0.0                                   # Dirichlet faces carry no flux row
    scale = np.abs(flux).max()
    assert np.abs(rx).max() < 1e-9 * scale
