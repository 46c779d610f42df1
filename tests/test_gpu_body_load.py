"""Body loads on the GPU against the oracle's full collocation solve.

The reference's HPS body-load path does not run (reduce_body,
src_disc/hps_parallel_leaf_ops.py:94-100, names an undefined Nxc); its leaf
solve takes the body load at the interior nodes (:73-82).  The oracle
(oracle/adjoint.py: Collocation) solves the same discretisation without
eliminating anything: PDE rows with the body load at every leaf's interior
nodes, flux-balance rows at the interior faces.  Tolerance 1e-9 relative on the
leaf-node solution, as the other solve parity tests.
"""
import numpy as np
import pytest
import torch

from oracle import adjoint as oadjoint
from oracle import domain as odomain
from oracle import funcs as ofuncs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.fail('GPU tests need CUDA')
    from slablu_gb300 import build
    build.build()


def _body(xx):
    x = np.asarray(xx)
    return (200.0 * np.sin(7 * x[:, 0]) * np.cos(5 * x[:, 1]))[:, None]


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_domain_solver_body_load_matches_collocation_oracle(precision):
    import slablu_gb300 as sg
    p, n, kh = 8, 48, 30.0
    a = 1 / (2 * (n / (p - 2)))
    md = odomain.Multidomain([[0, 1], [0, 1]], a, p)
    part = odomain.SlabPartition(md, 1.0)
    co = md.coeffs(ofuncs.helmholtz_pdo(lambda x: ofuncs.bfield_gaussian_bumps(x, kh)))
    coll = oadjoint.Collocation(md, part, co)
    ud = lambda x: ofuncs.uu_dir_greens(np.asarray(x), kh)
    _, _, ref = coll.solve(ud(md.xx_active[part.I_Xtot]), _body(md.xx_tot))
    op = sg.pdo.PDO_2d(sg.pdo.ones, sg.pdo.ones, c=lambda xx: sg.built_in_funcs.bfield_gaussian_bumps(xx, kh))
    dom = sg.Domain_Solver(torch.tensor([[0, 1.0], [0, 1.0]]), op, kh, a, p=p, buf_constant=1.0,
                           precision=precision)
    dom.build('reduced_gpu', 'slabLU', verbose=False)
    sol, rel, _, _, _ = dom.solve(lambda xx: sg.built_in_funcs.uu_dir_func_greens(xx, kh),
                                  lambda xx: torch.as_tensor(_body(xx.cpu().numpy())))
    err = np.linalg.norm(sol.numpy() - ref) / np.linalg.norm(ref)
    assert err < 1e-9, err
    assert float(rel) < 1e-10
    # the body load changes the solution (the check above is not the no-load case)
    _, _, ref0 = coll.solve(ud(md.xx_active[part.I_Xtot]))
    assert np.linalg.norm(ref - ref0) > 1e-3 * np.linalg.norm(ref)
