"""The oracle's collocation system and adjoint gradient (CPU).

Pins oracle/adjoint.py two ways: its direct solve reproduces the DtN-based
oracle path (itself pinned to the reference's golden vectors), and its
gradients match central finite differences of that solve.
"""
import numpy as np
import pytest

from oracle import adjoint as oadj
from oracle import domain as odomain
from oracle import funcs as ofuncs


def _problem(p=6, n=16, kh=12.0, first_order=False, seed=0):
    a = 1 / (2 * (n / (p - 2)))
    md = odomain.Multidomain([[0, 1], [0, 1]], a, p)
    part = odomain.SlabPartition(md, 1.0)
    co = md.coeffs(ofuncs.helmholtz_pdo(lambda x: ofuncs.bfield_gaussian_bumps(x, kh)))
    if first_order:
        rng = np.random.default_rng(seed)
        co['c1'] = 0.3 * rng.standard_normal(co['c'].shape)
        co['c2'] = 0.3 * rng.standard_normal(co['c'].shape)
    u_dir = ofuncs.uu_dir_greens(md.xx_active[part.I_Xtot], kh).reshape(-1, 1)
    return md, part, co, u_dir


def test_collocation_solve_matches_dtn_oracle():
    md, part, co, u_dir = _problem()
    col = oadj.Collocation(md, part, co)
    uU, uf, sol = col.solve(u_dir)
    out = odomain.solve_full(md, part, co, lambda x: u_dir)
    assert np.linalg.norm(sol - out['sol_tot']) < 1e-9 * np.linalg.norm(out['sol_tot'])
    assert np.linalg.norm(uf - out['sol_faces']) < 1e-9 * np.linalg.norm(out['sol_faces'])


def _loss(md, part, co, u_dir, fbody, w):
    col = oadj.Collocation(md, part, co)
    _, _, sol = col.solve(u_dir, fbody)
    return float((w * sol).sum())


@pytest.mark.parametrize('first_order', [False, True])
def test_oracle_gradient_matches_finite_differences(first_order):
    md, part, co, u_dir = _problem(first_order=first_order)
    rng = np.random.default_rng(1)
    npts = md.nboxes * md.p ** 2
    w = rng.standard_normal((npts, 1))
    fbody = rng.standard_normal((npts, 1))
    col = oadj.Collocation(md, part, co)
    uU, uf, sol = col.solve(u_dir, fbody)
    g = col.gradient(uU, uf, w)
    checks = [k for k in oadj.KEYS if co.get(k) is not None]
    for key in checks:
        d = rng.standard_normal(co[key].shape)
        eps = 1e-6 * np.abs(co[key]).max() / np.abs(d).max()
        cp = dict(co); cp[key] = co[key] + eps * d
        cm = dict(co); cm[key] = co[key] - eps * d
        fd = (_loss(md, part, cp, u_dir, fbody, w) - _loss(md, part, cm, u_dir, fbody, w)) / (2 * eps)
        ad = float((g[key].reshape(d.shape) * d).sum())
        assert abs(fd - ad) <= 1e-6 * abs(fd) + 1e-12, (key, fd, ad)
    # Dirichlet data and body load enter linearly: a single difference is exact
    dd = rng.standard_normal(u_dir.shape)
    fd = (_loss(md, part, co, u_dir + dd, fbody, w) - _loss(md, part, co, u_dir - dd, fbody, w)) / 2
    assert abs(fd - float((g['bnd'] * dd).sum())) < 1e-8 * abs(fd)
    df = rng.standard_normal(fbody.shape)
    fd = (_loss(md, part, co, u_dir, fbody + df, w) - _loss(md, part, co, u_dir, fbody - df, w)) / 2
    assert abs(fd - float((g['lam_leaf'] * df).sum())) < 1e-8 * abs(fd)


def _mixed_problem(p=8, n=24, kh=12.0):
    """Helmholtz on the wavy annulus sector: coefficients c11, c22, c12, c2, c."""
    a = 1 / (2 * (n / (p - 2)))
    md = odomain.Multidomain([[0, 1], [0, 1]], a, p)
    part = odomain.SlabPartition(md, 1.0)
    pdo, pmap = ofuncs.curvy_annulus_pdo(kh, ofuncs.bfield_constant)
    co = md.coeffs(pdo)
    u_dir = ofuncs.uu_dir_greens(pmap(md.xx_active[part.I_Xtot]), kh).reshape(-1, 1)
    return md, part, co, u_dir


def test_collocation_with_mixed_derivative_matches_dtn_oracle():
    md, part, co, u_dir = _mixed_problem()
    assert co.get('c12') is not None
    col = oadj.Collocation(md, part, co)
    uU, uf, sol = col.solve(u_dir)
    out = odomain.solve_full(md, part, co, lambda x: u_dir)
    assert np.linalg.norm(sol - out['sol_tot']) < 1e-9 * np.linalg.norm(out['sol_tot'])
    assert np.linalg.norm(uf - out['sol_faces']) < 1e-9 * np.linalg.norm(out['sol_faces'])


def test_oracle_gradient_with_mixed_derivative_matches_finite_differences():
    md, part, co, u_dir = _mixed_problem()
    rng = np.random.default_rng(3)
    npts = md.nboxes * md.p ** 2
    w = rng.standard_normal((npts, 1))
    fbody = rng.standard_normal((npts, 1))
    col = oadj.Collocation(md, part, co)
    uU, uf, sol = col.solve(u_dir, fbody)
    g = col.gradient(uU, uf, w)
    checks = [k for k in oadj.KEYS if co.get(k) is not None]
    assert 'c12' in checks
    for key in checks:
        d = rng.standard_normal(co[key].shape)
        eps = 1e-6 * max(np.abs(co[key]).max(), 1.0) / np.abs(d).max()   # c1 may be zero everywhere
        cp = dict(co); cp[key] = co[key] + eps * d
        cm = dict(co); cm[key] = co[key] - eps * d
        fd = (_loss(md, part, cp, u_dir, fbody, w) - _loss(md, part, cm, u_dir, fbody, w)) / (2 * eps)
        ad = float((g[key].reshape(d.shape) * d).sum())
        assert abs(fd - ad) <= 1e-6 * abs(fd) + 1e-12, (key, fd, ad)
    dd = rng.standard_normal(u_dir.shape)
    fd = (_loss(md, part, co, u_dir + dd, fbody, w) - _loss(md, part, co, u_dir - dd, fbody, w)) / 2
    assert abs(fd - float((g['bnd'] * dd).sum())) < 1e-8 * abs(fd)
