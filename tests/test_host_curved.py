"""Host side of curved domains (CPU): Domain_Solver's coefficient fields for an
operator with a mixed derivative, the engine it asks for, and the driver's set-up
of the reference's curved-domain tests up to the GPU."""
import numpy as np
import pytest
import torch

import slablu_gb300 as sg
from oracle import domain, funcs


def _curvy(kh=20.0, box=((0, 6.0), (0, 1.0)), p=8, n=48):
    op, pmap, _ = sg.pdo.get_param_map_and_pdo('curvy_annulus', sg.built_in_funcs.bfield_constant, kh)
    a = 1 / (2 * (n / (p - 2)))
    return op, pmap, a


def test_domain_solver_coefficients_with_c12_match_oracle():
    kh, p, n = 20.0, 8, 48
    op, pmap, a = _curvy(kh, p=p, n=n)
    dom = sg.Domain_Solver(torch.tensor([[0, 6.0], [0, 1.0]]), op, kh, a, p=p, buf_constant=1.0, periodic_bc=True,
                           device='cpu')
    assert dom.mixed and dom.periodic_bc
    co = dom._coeffs()
    assert set(k for k, v in co.items() if v is not None) == {'c11', 'c22', 'c12', 'c1', 'c2', 'c'}
    md = domain.Multidomain([[0, 6.0], [0, 1.0]], a, p)
    pdo, _ = funcs.curvy_annulus_pdo(kh, funcs.bfield_constant)
    ref = md.coeffs(pdo)
    for k, v in co.items():
        r = ref[k].ravel()
        assert np.abs(v.numpy() - r).max() <= 1e-13 * max(np.abs(r).max(), 1.0), k


def test_engine_is_created_for_the_mixed_derivative(monkeypatch):
    made = {}

    class Stop(Exception):
        pass

    def fake_engine(geom, precision, mixed=False):
        made.update(precision=precision, mixed=mixed, p=geom.p)
        raise Stop

    import slablu_gb300.slablu_solver as ss
    monkeypatch.setattr(ss, 'SlabEngine', fake_engine)
    monkeypatch.setattr(ss.torch.cuda, 'synchronize', lambda *a, **k: None)
    kh = 20.0
    op, pmap, a = _curvy(kh)
    dom = sg.Domain_Solver(torch.tensor([[0, 6.0], [0, 1.0]]), op, kh, a, p=8, buf_constant=1.0, device='cpu')
    with pytest.raises(Stop):
        dom.build('reduced_gpu', 'slabLU', verbose=False)
    assert made == dict(precision='mixed', mixed=True, p=8)
    op_sq = sg.pdo.PDO_2d(sg.pdo.ones, sg.pdo.ones, c=lambda xx: sg.built_in_funcs.bfield_constant(xx, kh))
    dom = sg.Domain_Solver(torch.tensor([[0, 1.0], [0, 1.0]]), op_sq, kh, a, p=8, buf_constant=1.0, device='cpu')
    with pytest.raises(Stop):
        dom.build('reduced_gpu', 'slabLU', verbose=False)
    assert made['mixed'] is False


def test_driver_sets_up_the_reference_curved_tests(monkeypatch):
    """argparse_driver with the reference tests' arguments reaches the solver with the
    curved-domain operator, the periodic partition and boundary data at mapped points."""
    from slablu_gb300 import argparse_driver
    seen = {}

    class Stop(Exception):
        pass

    class FakeSolver:
        def __init__(self, box_geom, op, kh, a, p=0, buf_constant=0.5, periodic_bc=False, precision='mixed', tol=1e-10):
            seen.update(box=np.asarray(box_geom), c12=op.c12 is not None, kh=kh, a=a, p=p, periodic=periodic_bc)
            raise Stop

    monkeypatch.setattr(argparse_driver, 'Domain_Solver', FakeSolver)
    with pytest.raises(Stop):
        argparse_driver.main(['--n', '400', '--pde', 'bfield_constant', '--bc', 'free_space', '--disc', 'hps',
                              '--p', '22', '--domain', 'curvy_annulus', '--ppw', '40', '--box_xlim', '6.0',
                              '--periodic_bc'])
    assert seen['c12'] and seen['periodic'] and seen['p'] == 22
    assert np.array_equal(seen['box'], [[0, 6.0], [0, 1.0]])
    assert abs(seen['kh'] - ((10 + 0.03) * 2 * np.pi + 1.8)) < 1e-12 and abs(seen['a'] - 1 / 40) < 1e-15
    with pytest.raises(ValueError):
        argparse_driver.main(['--n', '400', '--pde', 'bfield_constant', '--bc', 'free_space', '--disc', 'hps',
                              '--p', '22', '--domain', 'corner', '--ppw', '40'])


def test_driver_pickles_the_reference_keys(monkeypatch, tmp_path):
    """The driver writes two pickles, build_info then solve_info, with the keys the
    reference's driver writes (argparse_driver.py:169-188, 248-298)."""
    import pickle
    from slablu_gb300 import argparse_driver

    class SolverDouble:
        def __init__(self, box_geom, op, kh, a, p=0, buf_constant=0.5, periodic_bc=False, precision='mixed',
                     tol=1e-10):
            self.hps = type('H', (), {'n': torch.tensor([4, 4]), 'xx_tot': torch.zeros(16 * p * p, 2)})()
            self.buf_pans = 2
            self.last_solve_info = dict(iters=3)

        def build(self, sparse_assembly, solver_type, verbose=True):
            return dict(toc_build=0.5, toc_assembly=0.1, toc_factor=0.4, mem_build=1.0, precision='mixed')

        def solve(self, uu_dir, ff_body, known_sol=False):
            return torch.zeros(1, 1), torch.tensor(1e-12), torch.tensor(1e-9), 1e-10, 0.25

    monkeypatch.setattr(argparse_driver, 'Domain_Solver', SolverDouble)
    out = tmp_path / 'res.pkl'
    argparse_driver.main(['--n', '80', '--pde', 'bfield_constant', '--bc', 'free_space', '--disc', 'hps', '--p', '12',
                          '--domain', 'square', '--ppw', '10', '--pickle', str(out)])
    with open(out, 'rb') as f:
        build_info = pickle.load(f)
        solve_info = pickle.load(f)
    for k in ('toc_build', 'mem_build', 'toc_assembly', 'N', 'n', 'disc', 'buf', 'pde', 'bc', 'domain', 'solver',
              'sparse_assembly', 'box_geom', 'kh', 'periodic_bc', 'a', 'p'):
        assert k in build_info, k
    for k in ('res_solve', 'trueres_solve', 'resloc_hps_solve', 'toc_solve'):
        assert k in solve_info, k
    assert build_info['N'] == 10 * (12 * 16 + 4 + 4) and build_info['buf'] == 2 * 10
