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
import functools
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


@functools.lru_cache(maxsize=None)
class _CpuLU:
    """Test double of periodic.DenseLU for CPU tensors (the product factors the edge
    Schur complement on the GPU with the library's LU)."""

    def __init__(self, S):
        self.lu, self.piv = torch.linalg.lu_factor(S)

    def solve(self, B):
        return torch.linalg.lu_solve(self.lu, self.piv, B)


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
    edge = periodic.PeriodicEdge(eng, flux, left, right, geom.ntot, chunk=64, dense_lu=_CpuLU).build('cpu')
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
    # a body load would need its particular flux in the edge balance: refused
    with pytest.raises(NotImplementedError):
        edge.solve(bnd, fbody=torch.zeros(md.nboxes * md.p ** 2, 1, dtype=torch.float64))


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


@pytest.mark.parametrize('name', [NAME, 'periodic_curvy_annulus_p12_n230.npz'])
def test_domain_solver_periodic_flow_on_cpu(golden_dir, monkeypatch, name):
    """Domain_Solver(periodic_bc=True) end to end with the GPU pieces replaced by CPU
    doubles (the engine's non-periodic solve by a sparse direct solve, the reduced
    operator by the oracle's assembly and torch's CSR product): build, the periodic
    solve, the folded right-hand side and the folded residual are the product's code."""
    import slablu_gb300 as sg
    import slablu_gb300.slablu_solver as ss
    g, geom, md, part, co, A, ud = _setup(golden_dir, name)
    kh = float(g['kh'])
    curvy = 'curvy' in name
    As = A.copy()
    As.sort_indices()

    class EngineDouble(NonPeriodicSolveDouble):
        def __init__(self, geom_, precision, mixed=False):
            assert mixed == curvy
            super().__init__(md, part, A, co)
            self.factor_bytes = 0

        def factor(self, **coeffs):
            self.factored = sorted(k for k, v in coeffs.items() if v is not None)

    def sparse_mat(view, device='cuda', verbose=False):
        R = sparse.ReducedCSR(torch.as_tensor(As.indptr, dtype=torch.int64),
                              torch.as_tensor(As.indices, dtype=torch.int32),
                              torch.as_tensor(As.data), (geom.ntot, geom.ntot))
        view._A = R
        return R.to_torch(), {}

    def matvec(self, x, alpha=1.0, beta=0.0, y=None):
        X = x[:, None] if x.dim() == 1 else x
        M = torch.sparse_csr_tensor(self.indptr, self.indices.to(torch.int64), self.vals, size=self.shape)
        out = alpha * (M @ X.contiguous())
        return out[:, 0] if x.dim() == 1 else out

    monkeypatch.setattr(ss, 'SlabEngine', EngineDouble)
    monkeypatch.setattr(ss.periodic, 'DenseLU', _CpuLU)
    monkeypatch.setattr(ss._HPSView, 'sparse_mat', sparse_mat)
    monkeypatch.setattr(sparse.ReducedCSR, 'matvec', matvec)
    monkeypatch.setattr(ss.torch.cuda, 'synchronize', lambda *a, **k: None)
    p, n = int(g['p']), int(g['n'])
    if curvy:
        op, pmap, _ = sg.pdo.get_param_map_and_pdo('curvy_annulus', sg.built_in_funcs.bfield_constant, kh)
    else:
        op = sg.pdo.PDO_2d(sg.pdo.ones, sg.pdo.ones, c=lambda xx: sg.built_in_funcs.bfield_gaussian_bumps(xx, kh))
        pmap = lambda xx: xx
    dom = sg.Domain_Solver(torch.tensor(g['box']), op, kh, 1 / (2 * (n / (p - 2))), p=p, buf_constant=1.0,
                           periodic_bc=True, device='cpu')
    info = dom.build('reduced_gpu', 'slabLU', verbose=False)
    assert info['periodic_edge_size'] == g['I_Ctot_copy1'].size
    assert dom.engine.factored == (['c', 'c1', 'c11', 'c12', 'c2', 'c22'] if curvy else ['c', 'c11', 'c22'])
    uu = lambda xx: sg.built_in_funcs.uu_dir_func_greens(pmap(xx), kh)
    sol, res, tres, rloc, _ = dom.solve(uu, None, known_sol=True)
    stride = int(g['stride'])
    ref = g['superLU_sol_sub']
    assert np.linalg.norm(sol.numpy()[::stride] - ref) / np.linalg.norm(ref) < 1e-10
    assert float(res) < 1e-12
    assert abs(float(tres) - float(g['superLU_trueres'])) < 1e-8 * float(g['superLU_trueres'])
    ff = dom.get_rhs(uu)
    n_unique = g['I_Ctot_unique'].size if 'I_Ctot_unique' in g.files else int(g['I_Ctot_unique_size'])
    assert ff.shape[0] == n_unique
    ffr = domain.dirichlet_rhs(A, domain.SlabPartition(md, 1.0, periodic=True),
                               ud(md.xx_active[dom.I_Xtot.numpy()]).reshape(-1, 1))
    assert np.linalg.norm(ff.numpy() - ffr) <= 1e-12 * np.linalg.norm(ffr)
    with pytest.raises(NotImplementedError):
        dom.solve(uu, lambda xx: torch.ones(xx.shape[0], 1, dtype=torch.float64))
