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
