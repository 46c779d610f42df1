"""Periodic boundary: the oracle against the reference's own results.

Domain_Solver(periodic_bc=True) identifies the left and right edges of the
rectangle (the left edge of slab 0 with the right edge of the last slab) and
takes Dirichlet data on the bottom and top only.  The fixtures were written by
tests/golden/make_golden.py with the reference itself: the curvy annulus of the
reference's third test (tests/test_2d.py:54-55; parameter map with a mixed
derivative, rectangle [0, 6] x [0, 1] wrapping once around the origin) at a
smaller size, and Helmholtz with Gaussian bumps on a periodic unit square.  Both
the reference's superLU path (folded sparse matrix) and its slabLU path (cyclic
interface solver, HBS-compressed interface blocks) are recorded.
"""
import hashlib
import os

import numpy as np
import pytest

from oracle import block_tridiag as bt
from oracle import domain, funcs

CASES = ['periodic_square_p12_n210.npz', 'periodic_curvy_annulus_p12_n230.npz']


def _problem(g, name):
    p, n, kh = int(g['p']), int(g['n']), float(g['kh'])
    a = 1 / (2 * (n / (p - 2)))
    md = domain.Multidomain(g['box'], a, p)
    part = domain.SlabPartition(md, 1.0, periodic=True)
    if 'curvy' in name:
        pdo, pmap = funcs.curvy_annulus_pdo(kh, funcs.bfield_constant)
    else:
        pdo = funcs.helmholtz_pdo(lambda x: funcs.bfield_gaussian_bumps(x, kh))
        pmap = lambda x: x
    ud = lambda x: funcs.uu_dir_greens(pmap(x), kh)
    return md, part, pdo, pmap, ud


def _check_index(g, part, nm):
    v = np.ascontiguousarray(getattr(part, nm), dtype=np.int64)
    if nm in g.files:
        assert np.array_equal(v, g[nm]), nm
    else:
        assert v.size == int(g[nm + '_size']), nm
        assert hashlib.sha256(v.tobytes()).hexdigest() == str(g[nm + '_sha256']), nm


@pytest.mark.parametrize('name', CASES)
def test_periodic_partition_and_superlu(golden_dir, name):
    g = np.load(os.path.join(golden_dir, name))
    md, part, pdo, pmap, ud = _problem(g, name)
    assert (part.buf, part.Npan) == (int(g['buf']), int(g['Npan']))
    assert np.array_equal([md.n0, md.n1], g['nbox'])
    for nm in ('I_Ctot', 'I_Xtot', 'I_slabX', 'I_Ctot_unique', 'I_Ctot_copy1', 'I_Ctot_copy2'):
        _check_index(g, part, nm)
    if 'coef_xx' in g.files:
        xs = g['coef_xx']
        assert np.abs(pmap(xs) - g['mapped_xx']).max() < 1e-14
        for k in ('c11', 'c22', 'c12', 'c1', 'c2', 'c'):
            ref = g['coef_' + k]
            if k not in pdo:
                assert np.abs(ref).max() == 0.0, k
                continue
            assert np.abs(pdo[k](xs) - ref).max() <= 1e-13 * max(np.abs(ref).max(), 1.0), k
    co = md.coeffs(pdo)
    out = domain.solve_full(md, part, co, ud)
    sol = out['sol_tot']
    stride = int(g['stride'])
    ref = g['superLU_sol_sub']
    assert np.linalg.norm(sol[::stride] - ref) / np.linalg.norm(ref) < 1e-10
    assert abs(np.linalg.norm(sol) - float(g['superLU_sol_norm'])) < 1e-10 * float(g['superLU_sol_norm'])
    assert out['res'] < 1e-12
    true = ud(md.xx_tot)
    trueres = np.linalg.norm(sol - true) / np.linalg.norm(true)
    assert abs(trueres - float(g['superLU_trueres'])) < 1e-6 * float(g['superLU_trueres'])
    # the right edge carries the left edge's values
    fs = out['sol_faces']
    assert np.array_equal(fs[part.I_Ctot[part.I_Ctot_copy2]], fs[part.I_Ctot[part.I_Ctot_copy1]])
    # the reference's slabLU (HBS-compressed interface blocks) agrees with its superLU
    refs = g['slabLU_sol_sub']
    assert np.linalg.norm(sol[::stride] - refs) / np.linalg.norm(refs) < 1e-8


def test_periodic_slablu_cyclic_interface(golden_dir):
    """Two-level slab solver with the cyclic interface system on the periodic
    square: the same reduced solution as the folded sparse direct solve."""
    name = CASES[0]
    g = np.load(os.path.join(golden_dir, name))
    md, part, pdo, pmap, ud = _problem(g, name)
    co = md.coeffs(pdo)
    A = md.sparse_mat(domain.leafmod.dtn_build(md.ld, co))
    u_dir = ud(md.xx_active[part.I_Xtot]).reshape(-1, 1)
    x_direct, ff, _ = domain.solve_superlu(md, part, A, u_dir)
    S = domain.SlabLU(md, part, A)
    x = S.solve(domain.dirichlet_rhs(A, part, u_dir, fold=False))
    assert np.linalg.norm(x - x_direct) / np.linalg.norm(x_direct) < 1e-10
    sol = domain.assemble_solution(md, part, x, u_dir)
    u_tot, _ = domain.leaf_recover(md, co, sol)
    stride = int(g['stride'])
    refs = g['slabLU_sol_sub']
    assert np.linalg.norm(u_tot[::stride] - refs) / np.linalg.norm(refs) < 1e-8


def test_cyclic_block_lu_dense():
    """The cyclic interface solver against a dense solve of the wrapped matrix."""
    rng = np.random.default_rng(3)
    for nb, n in ((3, 4), (5, 6), (8, 3)):
        diag = rng.standard_normal((nb, n, n)) + 4 * n * np.eye(n)
        sub = rng.standard_normal((nb, n, n))
        sup = rng.standard_normal((nb, n, n))
        M = np.zeros((nb * n, nb * n))
        for j in range(nb):
            blk = lambda i: slice(i * n, (i + 1) * n)
            M[blk(j), blk(j)] = diag[j]
            M[blk(j), blk((j - 1) % nb)] = sub[j]
            M[blk(j), blk((j + 1) % nb)] = sup[j]
        f = rng.standard_normal((nb, n, 2))
        x = bt.CyclicInterfaceBlockLU(diag, sub, sup).solve(f)
        xd = np.linalg.solve(M, f.reshape(nb * n, 2)).reshape(nb, n, 2)
        assert np.abs(x - xd).max() < 1e-12 * np.abs(xd).max()
    with pytest.raises(ValueError):
        bt.CyclicInterfaceBlockLU(diag[:2], sub[:2], sup[:2])
