"""Periodic boundary on the GPU: Domain_Solver(periodic_bc=True) against the
reference's periodic solution.

Fixture: tests/golden/periodic_square_p12_n210.npz, made by the reference
itself (its superLU path on the folded sparse matrix, and its slabLU path with
the cyclic interface solver): Helmholtz with Gaussian bumps on the unit square,
left and right edges identified, free-space Green's function data on the
bottom and top, p = 12, 21 x 21 leaves, 7 slabs.  Tolerance: 1e-9 relative on
the leaf-node solution (the engine refines every solve to 1e-10 relative
correction, as in the non-periodic parity tests).  The folded reduced residual
(the reference's rel_err) is bounded by 1e-8: it is the residual of the reduced
system assembled from separately computed FP64 leaf DtN maps, so it carries
their rounding times the reduced operator's conditioning.
"""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NAME = 'periodic_square_p12_n210.npz'


@pytest.fixture(scope='module', autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.fail('GPU tests need CUDA')
    from slablu_gb300 import build
    build.build()


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_domain_solver_periodic_matches_reference(golden_dir, precision):
    import slablu_gb300 as sg
    g = np.load(os.path.join(golden_dir, NAME))
    p, n, kh = int(g['p']), int(g['n']), float(g['kh'])
    a = 1 / (2 * (n / (p - 2)))
    op = sg.pdo.PDO_2d(sg.pdo.ones, sg.pdo.ones, c=lambda xx: sg.built_in_funcs.bfield_gaussian_bumps(xx, kh))
    dom = sg.Domain_Solver(torch.tensor(g['box']), op, kh, a, p=p, buf_constant=1.0, periodic_bc=True,
                           precision=precision)
    assert (dom.buf_pans, dom.Npan) == (int(g['buf']), int(g['Npan']))
    for nm in ('I_Ctot', 'I_Xtot', 'I_slabX', 'I_Ctot_unique', 'I_Ctot_copy1', 'I_Ctot_copy2'):
        assert np.array_equal(getattr(dom, nm).numpy(), g[nm]), nm
    info = dom.build('reduced_gpu', 'slabLU', verbose=False)
    assert info['periodic_edge_size'] == g['I_Ctot_copy1'].size
    uu = lambda xx: sg.built_in_funcs.uu_dir_func_greens(xx, kh)
    sol, res, tres, rloc, toc = dom.solve(uu, None, known_sol=True)
    stride = int(g['stride'])
    ref = g['superLU_sol_sub']
    err = np.linalg.norm(sol.numpy()[::stride] - ref) / np.linalg.norm(ref)
    assert err < 1e-9, err
    assert float(res) < 1e-8, float(res)
    assert abs(float(tres) - float(g['superLU_trueres'])) < 1e-6 * float(g['superLU_trueres'])
    assert dom.last_solve_info['edge_rel_residual'] < 1e-6
    # folded right-hand side on the unique unknowns (get_rhs with sum_body_load)
    ff = dom.get_rhs(uu)
    assert ff.shape[0] == g['I_Ctot_unique'].size
    ffu = dom.get_rhs(uu, sum_body_load=False)
    assert ffu.shape[0] == g['I_Ctot'].size
