"""Curved-domain parameter maps of the product (slablu_gb300.pdo) against the
reference's own coefficient values (fixtures written by the reference's
pdo.get_param_map_and_pdo, tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest
import torch

from slablu_gb300 import pdo

KH_FIXTURES = [('annulus', 'annulus_p22_n400_ppw40.npz'),
               ('curvy_annulus', 'periodic_curvy_annulus_p12_n230.npz')]


def _bfield_constant(xx, kh):
    return -(kh ** 2) * torch.ones(xx.shape[0], dtype=torch.float64)


@pytest.mark.parametrize('geom,name', KH_FIXTURES)
def test_parameter_map_coefficients_match_reference(golden_dir, geom, name):
    g = np.load(os.path.join(golden_dir, name))
    kh = float(g['kh'])
    op, pmap, inv = pdo.get_param_map_and_pdo(geom, _bfield_constant, kh)
    xs = torch.as_tensor(g['coef_xx'])
    assert np.abs(pmap(xs).numpy() - g['mapped_xx']).max() < 1e-14
    # the inverse map recovers x1 modulo 6 (one turn: theta = x1 pi / 3, atan2 in (-pi, pi])
    back = inv(pmap(xs)).numpy() - g['coef_xx']
    back[:, 0] = (back[:, 0] + 3.0) % 6.0 - 3.0
    assert np.abs(back).max() < 1e-12
    for k in ('c11', 'c22', 'c12', 'c1', 'c2', 'c'):
        ref = g['coef_' + k]
        f = getattr(op, k)
        if f is None:
            assert np.abs(ref).max() == 0.0, k
            continue
        assert np.abs(f(xs).numpy() - ref).max() <= 1e-13 * max(np.abs(ref).max(), 1.0), k


def test_square_and_unknown_geometry():
    op, pmap, inv = pdo.get_param_map_and_pdo('square', _bfield_constant, 3.0)
    xs = torch.rand(7, 2, dtype=torch.float64)
    assert op.c12 is None and torch.equal(pmap(xs), xs) and torch.equal(inv(xs), xs)
    assert torch.allclose(op.c(xs), torch.full((7,), -9.0, dtype=torch.float64))
    op, pmap, inv = pdo.get_param_map_and_pdo('curved', _bfield_constant, 3.0)
    assert op.c12 is not None and op.c1 is None
    assert torch.allclose(inv(pmap(xs)), xs, atol=1e-14)
    with pytest.raises(ValueError):
        pdo.get_param_map_and_pdo('corner', _bfield_constant, 3.0)


@pytest.mark.parametrize('geom', ['curved', 'annulus', 'curvy_annulus'])
def test_every_parameter_map_matches_reference(golden_dir, geom):
    """All three curved domains of the reference (the sinusoidal strip included), product
    (torch) and oracle (NumPy), at seeded points (tests/golden/param_maps.npz)."""
    from oracle import funcs
    g = np.load(os.path.join(golden_dir, 'param_maps.npz'))
    kh = float(g['kh'])
    xs = g[geom + '_xx']
    op, pmap, _ = pdo.get_param_map_and_pdo(geom, _bfield_constant, kh)
    opo, pmapo = funcs.param_pdo(geom, kh, funcs.bfield_constant)
    assert np.abs(pmap(torch.as_tensor(xs)).numpy() - g[geom + '_mapped']).max() < 1e-14
    assert np.abs(pmapo(xs) - g[geom + '_mapped']).max() < 1e-14
    for k in ('c11', 'c22', 'c12', 'c1', 'c2', 'c'):
        ref = g[geom + '_' + k]
        tol = 1e-13 * max(np.abs(ref).max(), 1.0)
        f = getattr(op, k)
        fo = opo.get(k)
        if f is None:
            assert np.abs(ref).max() == 0.0 and fo is None, k
            continue
        assert np.abs(f(torch.as_tensor(xs)).numpy() - ref).max() <= tol, k
        assert np.abs(fo(xs) - ref).max() <= tol, k
