"""Pin the CPU oracle to golden vectors produced by the reference itself.

The fixtures in tests/golden/ were written by tests/golden/make_golden.py,
which runs the unmodified reference (annayesy/slabLU).  Integer/index data
must match exactly; FP64 data to a few ulps of the operator scale.
"""
import os

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import block_tridiag as bt
from oracle import domain, funcs, leaf


def load(golden_dir, name):
    return np.load(os.path.join(golden_dir, name))


@pytest.mark.parametrize('p', [8, 12, 22, 16])
def test_leaf_discretisation(golden_dir, p):
    g = load(golden_dir, f'leaf_p{p}.npz')
    ld = leaf.leaf_disc(float(g['a']), p)
    for nm in ('Jl', 'Jr', 'Jd', 'Ju', 'Jx', 'Jc', 'Jxreorder'):
        assert np.array_equal(getattr(ld, nm), g[nm]), nm
    assert np.array_equal(ld.zz, g['zz'])
    scale = np.abs(g['Nx']).max()
    assert np.abs(ld.Nx - g['Nx']).max() <= 1e-14 * scale
    assert np.abs(ld.Interp_mat - g['Interp_mat']).max() <= 1e-10
    if 'D11' in g:
        for nm in ('D1', 'D2', 'D11', 'D22'):
            assert np.abs(getattr(ld, nm) - g[nm]).max() <= 1e-14 * np.abs(g[nm]).max(), nm


@pytest.mark.parametrize('name', ['dtn_p22.npz', 'dtn_p12.npz'])
def test_leaf_dtn_build_and_solve(golden_dir, name):
    g = load(golden_dir, name)
    p = int(g['p'])
    ld = leaf.leaf_disc(float(g['a']), p)
    n = g['c'].shape[0]
    co = {'c11': np.ones((n, p * p)), 'c22': np.ones((n, p * p)), 'c': g['c']}
    dtn = leaf.dtn_build(ld, co)
    rel = np.linalg.norm(dtn - g['dtn'], axis=(1, 2)) / np.linalg.norm(g['dtn'], axis=(1, 2))
    assert rel.max() < 1e-12
    u, res = leaf.dtn_solve(ld, co, g['u_face'])
    nrhs = g['u_face'].shape[-1]
    ref_u = g['u_solve'][..., :nrhs]
    ref_res = g['u_solve'][..., nrhs:]
    assert np.linalg.norm(u - ref_u) / np.linalg.norm(ref_u) < 1e-12
    assert np.abs(res - ref_res).max() < 1e-6 * np.abs(ref_u).max() * np.abs(g['c']).max()


@pytest.mark.parametrize('name', ['dtn_c12_p12.npz', 'dtn_c12_p8.npz'])
def test_leaf_dtn_with_mixed_derivative(golden_dir, name):
    """Every coefficient present, c12 included: the reference's Jxreorder / Interp_mat
    branch of form_DtNs (hps_parallel_leaf_ops.py:59-65, 84-88)."""
    g = load(golden_dir, name)
    p = int(g['p'])
    ld = leaf.leaf_disc(float(g['a']), p)
    co = {k: g[k] for k in ('c11', 'c22', 'c12', 'c1', 'c2', 'c')}
    dtn = leaf.dtn_build(ld, co)
    rel = np.linalg.norm(dtn - g['dtn'], axis=(1, 2)) / np.linalg.norm(g['dtn'], axis=(1, 2))
    assert rel.max() < 1e-12, rel.max()
    u, res = leaf.dtn_solve(ld, co, g['u_face'])
    nrhs = g['u_face'].shape[-1]
    ref_u = g['u_solve'][..., :nrhs]
    ref_res = g['u_solve'][..., nrhs:]
    assert np.linalg.norm(u - ref_u) / np.linalg.norm(ref_u) < 1e-12
    assert np.abs(res - ref_res).max() < 1e-6 * np.abs(ref_u).max() * np.abs(g['c']).max()


def test_sparse_assembly(golden_dir):
    g = load(golden_dir, 'assembly_p8.npz')
    p, a, kh = int(g['p']), float(g['a']), float(g['kh'])
    md = domain.Multidomain(g['box_geom'], a, p)
    assert np.array_equal(md.I_unique, g['I_unique'])
    assert np.array_equal(md.I_copy1, g['I_copy1'])
    assert np.array_equal(md.I_copy2, g['I_copy2'])
    assert np.allclose(md.xx_active, g['xx_active'], rtol=0, atol=1e-15)
    co = md.coeffs(funcs.helmholtz_pdo(lambda x: funcs.bfield_gaussian_bumps(x, kh)))
    A = md.sparse_mat(leaf.dtn_build(md.ld, co))
    A.sort_indices()
    Ag = sp.csr_matrix((g['data'], g['indices'], g['indptr']), shape=tuple(g['shape']))
    assert np.array_equal(A.indptr, Ag.indptr) and np.array_equal(A.indices, Ag.indices)
    assert np.abs(A.data - Ag.data).max() <= 1e-13 * np.abs(Ag.data).max()


@pytest.mark.parametrize('p,n', [(8, 48), (12, 400), (22, 400), (22, 2000), (22, 1000), (16, 994)])
def test_slab_partition(golden_dir, p, n):
    g = load(golden_dir, 'partition.npz')
    tag = f'p{p}_n{n}'
    a = 1 / (2 * (n / (p - 2)))
    md = domain.Multidomain.__new__(domain.Multidomain)
    md.q = p - 2
    md.n0, md.n1 = [int(v) for v in g[tag + '_nbox']]
    part = domain.SlabPartition(md, 1.0)
    assert part.buf == int(g[tag + '_buf']) and part.Npan == int(g[tag + '_Npan'])
    for nm in ('I_C', 'I_L', 'I_R', 'I_D', 'I_U', 'I_Ctot', 'I_Xtot'):
        assert np.array_equal(getattr(part, nm), g[tag + '_' + nm]), nm
    ntot = md.q * (md.n0 * (2 * md.n1 + 1) + md.n1)
    assert np.array_equal(np.sort(np.concatenate((part.I_Ctot, part.I_Xtot))), np.arange(ntot))
    del a


@pytest.mark.parametrize('tag', ['b3_m5_bs4', 'b2_m7_bs6', 'b4_m2_bs3'])
def test_block_tridiag(golden_dir, tag):
    g = load(golden_dir, 'blocktri.npz')
    T = bt.BlockTridiag(g[tag + '_diag'], g[tag + '_sub'], g[tag + '_sup'])
    assert np.array_equal(T.piv + 1, g[tag + '_piv'])
    for nm, mine in (('LU', T.LU), ('Lsub', T.Lsub), ('Usup', T.Usup)):
        assert np.abs(mine - g[tag + '_' + nm]).max() < 1e-12, nm
    x = T.solve(g[tag + '_f'])
    xt = T.solve(g[tag + '_f'], transpose=True)
    assert np.abs(x - g[tag + '_x']).max() < 1e-11
    assert np.abs(xt - g[tag + '_xt']).max() < 1e-11
    assert np.abs(T.matvec(x) - g[tag + '_f']).max() < 1e-10
    assert np.abs(T.matvec(xt, transpose=True) - g[tag + '_f']).max() < 1e-10


def test_superlu_solve_small(golden_dir):
    g = load(golden_dir, 'solve_superlu_p8_n48.npz')
    p, n, kh = int(g['p']), int(g['n']), float(g['kh'])
    a = 1 / (2 * (n / (p - 2)))
    md = domain.Multidomain([[0, 1], [0, 1]], a, p)
    part = domain.SlabPartition(md, 1.0)
    co = md.coeffs(funcs.helmholtz_pdo(lambda x: funcs.bfield_gaussian_bumps(x, kh)))
    out = domain.solve_full(md, part, co, lambda x: funcs.uu_dir_greens(x, kh))
    assert np.linalg.norm(out['sol_tot'] - g['sol']) / np.linalg.norm(g['sol']) < 1e-12
    assert out['res'] < 1e-13
    # resloc is a roundoff-level absolute norm: compare orders of magnitude only
    assert 0.2 * float(g['resloc']) < out['resloc'] < 5 * float(g['resloc'])
    # the two-level slab solver reproduces the sparse direct solve
    S = domain.SlabLU(md, part, out['A'])
    x = S.solve(out['ff'])
    assert np.linalg.norm(x - out['x']) / np.linalg.norm(out['x']) < 1e-12


@pytest.mark.parametrize('name', ['slablu_p12_n400_ppw10.npz', 'slablu_p22_n400_ppw40.npz'])
def test_reference_slablu_solutions(golden_dir, name):
    """Known-answer test of the reference (tests/test_2d.py:43) and its solution vector."""
    g = load(golden_dir, name)
    p, n, kh = int(g['p']), int(g['n']), float(g['kh'])
    a = 1 / (2 * (n / (p - 2)))
    md = domain.Multidomain([[0, 1], [0, 1]], a, p)
    part = domain.SlabPartition(md, 1.0)
    co = md.coeffs(funcs.helmholtz_pdo(lambda x: funcs.bfield_constant(x, kh)))
    out = domain.solve_full(md, part, co, lambda x: funcs.uu_dir_greens(x, kh))
    sol = out['sol_tot']
    stride = int(g['stride'])
    assert np.linalg.norm(sol[::stride] - g['sol_sub']) / np.linalg.norm(g['sol_sub']) < 1e-9
    assert abs(np.linalg.norm(sol) - float(g['sol_norm'])) < 1e-9 * float(g['sol_norm'])
    true = funcs.uu_dir_greens(md.xx_tot, kh)
    trueres = np.linalg.norm(sol - true) / np.linalg.norm(true)
    assert abs(trueres - float(g['trueres'])) < 1e-6 * float(g['trueres']) + 1e-12
    if p == 22:
        assert trueres < 2e-5   # tests/test_2d.py:43 (p=22, n=400, ppw=40)


def test_reference_annulus_known_answer(golden_dir):
    """The reference's annulus test (tests/test_2d.py:51-52): Helmholtz on the annulus
    through its parameter map (coefficients with a mixed derivative), free-space
    Green's function data, trueres < 2e-5 (tests/test_2d.py:43), and the reference's
    solution vector."""
    g = load(golden_dir, 'annulus_p22_n400_ppw40.npz')
    p, n, kh = int(g['p']), int(g['n']), float(g['kh'])
    pdo, pmap = funcs.annulus_pdo(kh, funcs.bfield_constant)
    # the restated coefficient map against the reference's values at sampled nodes
    xs = g['coef_xx']
    assert np.abs(pmap(xs) - g['mapped_xx']).max() < 1e-14
    for k in ('c11', 'c22', 'c12', 'c2', 'c'):
        ref = g['coef_' + k]
        assert np.abs(pdo[k](xs) - ref).max() <= 1e-13 * max(np.abs(ref).max(), 1.0), k
    assert np.abs(g['coef_c1']).max() == 0.0
    a = 1 / (2 * (n / (p - 2)))
    md = domain.Multidomain([[0, 1], [0, 1]], a, p)
    part = domain.SlabPartition(md, 1.0)
    co = md.coeffs(pdo)
    ud = lambda x: funcs.uu_dir_greens(pmap(x), kh)
    out = domain.solve_full(md, part, co, ud)
    sol = out['sol_tot']
    stride = int(g['stride'])
    assert np.linalg.norm(sol[::stride] - g['sol_sub']) / np.linalg.norm(g['sol_sub']) < 1e-9
    true = ud(md.xx_tot)
    trueres = np.linalg.norm(sol - true) / np.linalg.norm(true)
    assert trueres < 2e-5
    assert abs(trueres - float(g['trueres'])) < 1e-3 * float(g['trueres'])


def test_reference_config1_plane_waves(golden_dir):
    """Config 1 (p = 12, n = 400, 10 points per wavelength): Dirichlet data a sum of
    8 seeded plane waves; the oracle's sparse direct solve against the reference's
    slabLU solution vector."""
    import torch
    from slablu_gb300 import problems
    g = load(golden_dir, 'config1_slabLU_p12_n400.npz')
    cfg = problems.config1()
    p, n, kh = int(g['p']), int(g['n']), float(g['kh'])
    assert (p, n) == (cfg['p'], cfg['n']) and kh == cfg['kh']
    md = domain.Multidomain([[0, 1], [0, 1]], cfg['a'], p)
    part = domain.SlabPartition(md, 1.0)
    co = md.coeffs(funcs.helmholtz_pdo(lambda x: funcs.bfield_constant(x, kh)))
    out = domain.solve_full(md, part, co, lambda x: cfg['uu_dir'](torch.as_tensor(x)).numpy())
    sol = out['sol_tot'][:, 0]
    stride = int(g['stride'])
    assert sol.size == int(g['sol_len'])
    assert np.linalg.norm(sol[::stride] - g['sol_sub']) / np.linalg.norm(g['sol_sub']) < 1e-9
    assert abs(np.linalg.norm(sol) - float(g['sol_norm'])) < 1e-9 * float(g['sol_norm'])


def test_reference_config2_leaf_dtn(golden_dir):
    """Config 2 (128 x 128 leaves, p = 22, 32-bump field): the oracle's leaf DtN maps
    against the reference's form_DtNs on the sampled leaves, and the sampled
    leaves' points and coefficients against the product's generators."""
    import torch
    from slablu_gb300 import hps, problems
    g = load(golden_dir, 'config2_dtn_p22.npz')
    cfg = problems.config2()
    p, a = int(g['p']), float(g['a'])
    assert p == cfg['p'] and a == cfg['a'] and int(g['nside']) == cfg['nside']
    geo = hps.Geometry([[0, 1], [0, 1]], a, p, 1.0)
    xx = np.asarray(geo.xx).reshape(-1, p * p, 2)[g['picks']]
    assert np.abs(xx - g['xx']).max() < 1e-15
    c = cfg['c'](torch.as_tensor(xx.reshape(-1, 2))).numpy().reshape(len(g['picks']), -1)
    assert np.array_equal(c, g['c'])
    ld = leaf.leaf_disc(a, p)
    n = c.shape[0]
    dtn = leaf.dtn_build(ld, {'c11': np.ones((n, p * p)), 'c22': np.ones((n, p * p)), 'c': g['c']})
    rel = np.linalg.norm(dtn - g['dtn'], axis=(1, 2)) / np.linalg.norm(g['dtn'], axis=(1, 2))
    assert rel.max() < 1e-12, rel.max()
