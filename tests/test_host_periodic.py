"""Host logic of the periodic boundary (slablu_gb300/periodic.py) on the CPU.

The GPU engine is replaced by a test double with the same solve() interface
that solves the non-periodic reduced system (both copies of the shared edge are
Dirichlet faces) with SciPy; the edge Schur complement, its correction steps,
the folded residual and the periodic index sets are the product's own code.
Checked against the reference's periodic solutions (tests/golden fixtures made by
the reference's superLU path): a periodic square with Gaussian bumps, and the
periodic curvy annulus of the reference's third test (mixed derivative; leaves
couple to their corners through Interp_mat) at a smaller size.
"""
import os

import numpy as np
import pytest
import scipy.sparse.linalg as spla
import torch

from oracle import domain, funcs, leaf as oleaf
from slablu_gb300 import periodic, sparse
from slablu_gb300.hps import Geometry

NAME = 'periodic_square_p12_n210.npz'


class NonPeriodicSolveDouble:
    """solve(bnd, fbody, tol, max_iter, want_faces, allow_noconv) of the engine,
    for the non-periodic partition, by a sparse direct solve."""

    def __init__(self, md, part, A, co):
        self.md, self.part, self.A, self.co = md, part, A, co
        self.lu = spla.splu(A[part.I_Ctot][:, part.I_Ctot].tocsc())
        self.A_CX = A[part.I_Ctot][:, part.I_Xtot]
        self.calls = []
        self.leaf_calls = 0

    def solve(self, bnd, fbody=None, tol=1e-10, max_iter=20, want_faces=False, allow_noconv=False, want_leaf=True):
        assert fbody is None
        b = bnd.numpy() if bnd.dim() == 2 else bnd.numpy()[:, None]
        self.calls.append(b.shape[1])
        uf = np.zeros_like(b)
        uf[self.part.I_Xtot] = b[self.part.I_Xtot]
        uf[self.part.I_Ctot] = self.lu.solve(-(self.A_CX @ b[self.part.I_Xtot]))
        u_leaf = torch.as_tensor(domain.leaf_recover(self.md, self.co, uf)[0]) if want_leaf else None
        self.leaf_calls += int(want_leaf)
        st = dict(rel_correction=0.0, residual=0.0, residual0=0.0, resloc=0.0, rel_residual=0.0, converged=True)
        return u_leaf, (torch.as_tensor(uf) if want_faces else None), 1, st


def _setup(golden_dir, name=NAME):
    g = np.load(os.path.join(golden_dir, name))
    p, n, kh = int(g['p']), int(g['n']), float(g['kh'])
    a = 1 / (2 * (n / (p - 2)))
    geom = Geometry(g['box'], a, p, 1.0)
    md = domain.Multidomain(g['box'], a, p)
    part = domain.SlabPartition(md, 1.0)                 # non-periodic: the engine's partition
    if 'curvy' in name:   # mixed derivative: the Jxreorder / Interp_mat leaf branch
        pdo, pmap = funcs.curvy_annulus_pdo(kh, funcs.bfield_constant)
    else:
        pdo, pmap = funcs.helmholtz_pdo(lambda x: funcs.bfield_gaussian_bumps(x, kh)), (lambda x: x)
    co = md.coeffs(pdo)
    A = md.sparse_mat(oleaf.dtn_build(md.ld, co)).tocsr()
    ud = lambda x: funcs.uu_dir_greens(pmap(x), kh)
    return g, geom, md, part, co, A, ud


def test_periodic_index_sets_of_the_reference_test(golden_dir):
    """The reference's third test at its own size (p = 22, n = 400, [0, 6] x [0, 1]):
    partition and periodic index sets (large sets by length and SHA-256)."""
    import hashlib
    g = np.load(os.path.join(golden_dir, 'periodic_curvy_annulus_p22_n400.npz'))
    p, n = int(g['p']), int(g['n'])
    geom = Geometry(g['box'], 1 / (2 * (n / (p - 2))), p, 1.0)
    assert (geom.buf, geom.Npan, geom.n0, geom.n1) == (int(g['buf']), int(g['Npan']), *map(int, g['nbox']))
    sets = periodic.periodic_index_sets(geom)
    for nm in ('I_Ctot', 'I_Xtot', 'I_slabX', 'I_Ctot_unique', 'I_Ctot_copy1', 'I_Ctot_copy2'):
        v = np.ascontiguousarray(sets[nm], dtype=np.int64)
        if nm in g.files:
            assert np.array_equal(v, g[nm]), nm
        else:
            assert v.size == int(g[nm + '_size']), nm
            assert hashlib.sha256(v.tobytes()).hexdigest() == str(g[nm + '_sha256']), nm


def test_periodic_index_sets_match_reference(golden_dir):
    g, geom, *_ = _setup(golden_dir)
    sets = periodic.periodic_index_sets(geom)
    for nm in ('I_Ctot', 'I_Xtot', 'I_slabX', 'I_Ctot_unique', 'I_Ctot_copy1', 'I_Ctot_copy2'):
        assert np.array_equal(sets[nm], g[nm]), nm
    left, right = periodic.edge_faces(geom)
    assert np.array_equal(sets['I_Ctot'][sets['I_Ctot_copy1']], left)
    assert np.array_equal(sets['I_Ctot'][sets['I_Ctot_copy2']], right)


@pytest.mark.parametrize('name', [NAME, 'periodic_curvy_annulus_p12_n230.npz'])
def test_periodic_edge_schur_solve(golden_dir, name):
    g, geom, md, part, co, A, ud = _setup(golden_dir, name)
    left, right = periodic.edge_faces(geom)
    rows = np.concatenate((left, right))
    Aedge = A[rows]
    flux = lambda U: torch.as_tensor(Aedge @ U.numpy())
    eng = NonPeriodicSolveDouble(md, part, A, co)
    edge = periodic.PeriodicEdge(eng, flux, left, right, geom.ntot, chunk=64).build('cpu')
    nL = left.size
    assert eng.calls[:(nL + 63) // 64] == [64] * (nL // 64) + ([nL % 64] if nL % 64 else [])
    sets = periodic.periodic_index_sets(geom)
    bnd = torch.zeros(geom.ntot, 1, dtype=torch.float64)
    bnd[sets['I_Xtot']] = torch.as_tensor(ud(geom.xx_active[sets['I_Xtot']]))
    u_leaf, uf, st = edge.solve(bnd)
    # the Schur columns and the zero-edge solve ask for face values only
    assert eng.leaf_calls == st['edge_steps']
    stride = int(g['stride'])
    ref = g['superLU_sol_sub']
    assert np.linalg.norm(u_leaf.numpy()[::stride] - ref) / np.linalg.norm(ref) < 1e-10
    assert st['edge_rel_residual'] < 1e-10
    # both copies of the edge carry the same values
    assert torch.equal(uf[left], uf[right])
    # folded reduced residual (the reference's rel_err of the periodic solve)
    ic = torch.as_tensor(sets['I_Ctot'])
    d = torch.zeros_like(uf)
    d[sets['I_Xtot']] = bnd[sets['I_Xtot']]
    Au = torch.as_tensor(A @ uf.numpy())
    Ad = torch.as_tensor(A @ d.numpy())
    r = periodic.fold(Au[ic], sets)
    ff = periodic.fold(-Ad[ic], sets)
    assert float(torch.linalg.norm(r) / torch.linalg.norm(ff)) < 1e-12


def test_fold_and_row_subset(golden_dir):
    g, geom, md, part, co, A, ud = _setup(golden_dir)
    sets = periodic.periodic_index_sets(geom)
    v = torch.arange(sets['I_Ctot'].size, dtype=torch.float64)[:, None]
    f = periodic.fold(v, sets)
    assert f.shape[0] == sets['I_Ctot_unique'].size
    c1, c2 = sets['I_Ctot_copy1'], sets['I_Ctot_copy2']
    assert torch.equal(f[c1, 0], v[c1, 0] + v[c2, 0])
    # row subset of the reduced operator shares its values
    indptr, indices, dest = sparse.reduced_pattern(geom)
    As = A.copy()
    As.sort_indices()
    assert np.array_equal(As.indptr, indptr) and np.array_equal(As.indices, indices)
    R = sparse.ReducedCSR(torch.as_tensor(indptr), torch.as_tensor(indices), torch.as_tensor(As.data),
                          (geom.ntot, geom.ntot))
    left, right = periodic.edge_faces(geom)
    rows = np.concatenate((left, right))
    E = sparse.row_subset(geom, R, rows)
    dense = E.to_torch().to_dense().numpy()
    assert np.array_equal(dense, As[rows].toarray())
