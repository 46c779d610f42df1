"""Curved domains on the GPU: operators with a mixed derivative (c12).

The reference solves on a curved domain by pulling Helmholtz back to a
rectangle through a parameter map (src_disc/pdo.py), which gives a c12 term,
and leaves then couple to their corners through Interp_mat
(src_disc/hps_parallel_leaf_ops.py:59-65, 84-92).  Checked here:
  * the engine (slab_engine_create_mixed) against the oracle's sparse direct
    solve of the same discretisation, given the same Interp_mat (1e-9);
  * Domain_Solver on the reference's own tests (tests/test_2d.py:51-55):
    the annulus and the periodic curvy annulus at the tests' sizes (and the
    latter smaller) against the reference's solutions, and both through the
    argparse driver with the tests' criterion trueres < 2e-5.
Tolerance against the reference's solutions: 1e-8, since the reference's
Interp_mat is an ill-conditioned least-squares fit whose last digits depend on
the LAPACK build (its face rows differ from the identity by ~1e-10).
"""
import os
import pickle

import numpy as np
import pytest
import torch

from oracle import domain as odomain
from oracle import funcs as ofuncs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.fail('GPU tests need CUDA')
    from slablu_gb300 import build
    build.build()


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_mixed_engine_matches_sparse_direct_oracle(precision):
    """Curvy-annulus coefficients (every term; |c12| up to 1: the map is not orthogonal,
    unlike the annulus's, whose c12 vanishes) on 8 x 8 leaves of order 8, two slabs."""
    from slablu_gb300 import hps
    from slablu_gb300.engine import SlabEngine
    p, n, kh = 8, 48, 12.0
    a = 1 / (2 * (n / (p - 2)))
    md = odomain.Multidomain([[0, 1], [0, 1]], a, p)
    part = odomain.SlabPartition(md, 1.0)
    g = hps.Geometry([[0, 1], [0, 1]], a, p, 1.0)
    md.ld.Interp_mat = np.array(g.ops.Interp_mat)     # the same fit on both sides
    pdo, pmap = ofuncs.curvy_annulus_pdo(kh, ofuncs.bfield_constant)
    co = md.coeffs(pdo)
    assert np.abs(co['c12']).max() > 0.5
    ud = lambda x: ofuncs.uu_dir_greens(pmap(x), kh)
    ref = odomain.solve_full(md, part, co, ud)['sol_tot']
    eng = SlabEngine(g, precision, mixed=True)
    eng.factor(**{k: (None if v is None else torch.as_tensor(v.ravel(), device='cuda')) for k, v in co.items()})
    bnd = torch.as_tensor(ud(md.xx_active), device='cuda')
    uleaf, _, iters, st = eng.solve(bnd, tol=1e-12, max_iter=30, want_faces=True)
    assert st['converged'], st
    err = np.linalg.norm(uleaf.cpu().numpy() - ref) / np.linalg.norm(ref)
    assert err < 1e-9, err
    # the engine refuses c12 without the mixed layout
    with pytest.raises(ValueError):
        SlabEngine(g, precision).factor(**{k: (None if v is None else torch.as_tensor(v.ravel(), device='cuda'))
                                           for k, v in co.items()})


def _annulus_solver(sg, geom, box, p, n, ppw, periodic, precision='mixed'):
    nwaves = int(n / ppw)
    kh = (nwaves + 0.03) * 2 * np.pi + 1.8
    op, pmap, _ = sg.pdo.get_param_map_and_pdo(geom, sg.built_in_funcs.bfield_constant, kh)
    a = 1 / (2 * (n / (p - 2)))
    dom = sg.Domain_Solver(torch.tensor(box), op, kh, a, p=p, buf_constant=1.0, periodic_bc=periodic,
                           precision=precision)
    dom.build('reduced_gpu', 'slabLU', verbose=False)
    uu = lambda xx: sg.built_in_funcs.uu_dir_func_greens(pmap(xx), kh)
    return dom, uu, kh


def test_domain_solver_annulus_matches_reference(golden_dir):
    """The reference's annulus test (p = 22, n = 400, ppw = 40) against its solution."""
    import slablu_gb300 as sg
    g = np.load(os.path.join(golden_dir, 'annulus_p22_n400_ppw40.npz'))
    dom, uu, kh = _annulus_solver(sg, 'annulus', [[0, 1.0], [0, 1.0]], int(g['p']), int(g['n']), int(g['ppw']),
                                  False)
    assert abs(kh - float(g['kh'])) < 1e-12
    sol, res, tres, rloc, _ = dom.solve(uu, None, known_sol=True)
    stride = int(g['stride'])
    err = np.linalg.norm(sol.numpy()[::stride] - g['sol_sub']) / np.linalg.norm(g['sol_sub'])
    assert err < 1e-8, err
    assert float(tres) < 2e-5
    assert float(res) < 1e-10


@pytest.mark.parametrize('name', ['periodic_curvy_annulus_p12_n230.npz', 'periodic_curvy_annulus_p22_n400.npz'])
def test_domain_solver_periodic_curvy_annulus_matches_reference(golden_dir, name):
    """The periodic curvy annulus: the reference's third test (p = 22, n = 400 on
    [0, 6] x [0, 1]) and a smaller case (p = 12, n = 230)."""
    import slablu_gb300 as sg
    g = np.load(os.path.join(golden_dir, name))
    dom, uu, kh = _annulus_solver(sg, 'curvy_annulus', g['box'].tolist(), int(g['p']), int(g['n']),
                                  int(g['ppw']), True)
    sol, res, tres, rloc, _ = dom.solve(uu, None, known_sol=True)
    stride = int(g['stride'])
    ref = g['superLU_sol_sub']
    err = np.linalg.norm(sol.numpy()[::stride] - ref) / np.linalg.norm(ref)
    assert err < 1e-8, err
    assert abs(float(tres) - float(g['superLU_trueres'])) < 1e-4 * float(g['superLU_trueres'])
    assert float(res) < 1e-8
    if int(g['p']) == 22:
        assert float(tres) < 2e-5   # the reference test's criterion (tests/test_2d.py:43)


@pytest.mark.parametrize('domain,extra', [('annulus', []), ('curvy_annulus', ['--box_xlim', '6.0', '--periodic_bc'])])
def test_reference_tests_through_the_driver(tmp_path, domain, extra):
    """tests/test_2d.py:8-55 of the reference, through this package's driver: HPS p = 22,
    n = 400, ppw = 40, constant Helmholtz, free-space data, trueres < 2e-5."""
    from slablu_gb300 import argparse_driver
    out = tmp_path / 'res.pkl'
    argparse_driver.main(['--n', '400', '--pde', 'bfield_constant', '--bc', 'free_space', '--pickle', str(out),
                          '--disc', 'hps', '--p', '22', '--domain', domain, '--ppw', '40', '--solver', 'slabLU',
                          '--sparse_assembly', 'reduced_gpu'] + extra)
    with open(out, 'rb') as f:
        _ = pickle.load(f)
        d = pickle.load(f)
    assert float(d['trueres_solve']) < 2e-5
