"""GPU adjoint: transposed solve with the stored factors and coefficient gradients.

Checked against (a) the dense FP64 reference gradient of the oracle's full
collocation system (oracle/adjoint.py, itself pinned to finite differences on
the CPU), with and without a mixed derivative c12, and (b) central finite differences of the GPU forward solve through
the torch.autograd.Function.  Tolerances: 1e-9 relative against the oracle
(FP64 refinement to 1e-12 on both sides of the solve); 1e-5 relative against
central differences.
"""
import numpy as np
import pytest
import torch

from oracle import adjoint as oadj
from oracle import domain as odomain
from oracle import funcs as ofuncs

pytestmark = pytest.mark.gpu

CASES = [
    ([[0, 1], [0, 1]], 8, 48, 30.0, False),    # 8 x 8 leaves, 2 slabs
    ([[0, 1], [0, 0.5]], 8, 48, 30.0, True),   # 8 x 4 leaves, first-order terms
    ([[0, 1], [0, 1]], 8, 72, 45.0, False),    # 12 x 12 leaves, 3 slabs
    ([[0, 1], [0, 1]], 22, 80, 30.0, False),   # p = 22 leaves, 4 x 4
]


@pytest.fixture(scope='module', autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.fail('GPU tests need CUDA')
    from slablu_gb300 import build
    build.build()


def _setup(case, precision):
    from slablu_gb300 import hps
    from slablu_gb300.engine import SlabEngine
    geom, p, n, kh, first = CASES[case]
    a = 1 / (2 * (n / (p - 2)))
    md = odomain.Multidomain(geom, a, p)
    part = odomain.SlabPartition(md, 1.0)
    co = md.coeffs(ofuncs.helmholtz_pdo(lambda x: ofuncs.bfield_gaussian_bumps(x, kh)))
    if first:
        rng = np.random.default_rng(7)
        co['c1'] = 5.0 * rng.standard_normal(co['c'].shape)
        co['c2'] = 5.0 * rng.standard_normal(co['c'].shape)
    g = hps.Geometry(geom, a, p, 1.0)
    eng = SlabEngine(g, precision)
    return md, part, co, eng, kh


def _dev(co):
    return {k: torch.as_tensor(v.ravel(), device='cuda') for k, v in co.items() if v is not None}


def _rel(x, y):
    return float(np.linalg.norm(x - y) / np.linalg.norm(y))


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
@pytest.mark.parametrize('case', range(len(CASES)))
def test_adjoint_matches_dense_reference_gradient(case, precision):
    md, part, co, eng, kh = _setup(case, precision)
    rng = np.random.default_rng(case)
    nrhs = 1
    B = rng.standard_normal((md.ntot, nrhs))
    w = rng.standard_normal((md.nboxes * md.p ** 2, nrhs))
    col = oadj.Collocation(md, part, co)
    uU, uf, sol = col.solve(B[part.I_Xtot])
    ref = col.gradient(uU, uf, w)
    eng.factor(**_dev(co))
    uleaf, ufaces, it, st = eng.solve(torch.as_tensor(B, device='cuda'), tol=1e-12, max_iter=40, want_faces=True)
    assert st['converged']
    assert _rel(uleaf.cpu().numpy(), sol) < 1e-9
    lam, lamf, gb, it_t, st_t = eng.adjoint(gleaf=torch.as_tensor(w, device='cuda'), tol=1e-12, max_iter=40,
                                            want_faces=True)
    assert st_t['converged'], st_t
    if precision == 'fp64':
        assert it_t <= 3
    assert _rel(lam.cpu().numpy(), ref['lam_leaf']) < 1e-9
    assert _rel(lamf.cpu().numpy(), ref['lam_faces']) < 1e-9
    gbn = gb.cpu().numpy()
    assert _rel(gbn[part.I_Xtot], ref['bnd']) < 1e-9
    nd = np.setdiff1d(np.arange(md.ntot), part.I_Xtot)
    assert np.abs(gbn[nd]).max() == 0.0
    keys = tuple(k for k in oadj.KEYS if co.get(k) is not None)
    grads = eng.coeff_grad(ufaces, uleaf, lam, keys=keys)
    for k in keys:
        assert _rel(grads[k].cpu().numpy(), ref[k]) < 1e-9, k


def _mixed_setup(precision):
    """Curvy-annulus coefficients (c11, c22, c12, c2, c; |c12| up to 1) on 8 x 8
    leaves of order 8: an engine with the mixed-derivative layout."""
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
    return md, part, co, SlabEngine(g, precision, mixed=True), kh


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_adjoint_with_mixed_derivative_matches_dense_reference_gradient(precision):
    """Transposed solve and coefficient gradients (dL/dc12 included) of an operator
    with c12 against the oracle's dense FP64 gradient, 1e-9 relative; the same
    gradients through slab_solve's backward."""
    from slablu_gb300 import slab_solve
    md, part, co, eng, kh = _mixed_setup(precision)
    rng = np.random.default_rng(21)
    nrhs = 2
    B = rng.standard_normal((md.ntot, nrhs))
    w = rng.standard_normal((md.nboxes * md.p ** 2, nrhs))
    col = oadj.Collocation(md, part, co)
    uU, uf, sol = col.solve(B[part.I_Xtot])
    ref = col.gradient(uU, uf, w)
    eng.factor(**_dev(co))
    uleaf, ufaces, it, st = eng.solve(torch.as_tensor(B, device='cuda'), tol=1e-12, max_iter=40, want_faces=True)
    assert st['converged']
    assert _rel(uleaf.cpu().numpy(), sol) < 1e-9
    lam, lamf, gb, it_t, st_t = eng.adjoint(gleaf=torch.as_tensor(w, device='cuda'), tol=1e-12, max_iter=40,
                                            want_faces=True)
    assert st_t['converged'], st_t
    if precision == 'fp64':
        assert it_t <= 3
    assert _rel(lam.cpu().numpy(), ref['lam_leaf']) < 1e-9
    assert _rel(lamf.cpu().numpy(), ref['lam_faces']) < 1e-9
    gbn = gb.cpu().numpy()
    assert _rel(gbn[part.I_Xtot], ref['bnd']) < 1e-9
    nd = np.setdiff1d(np.arange(md.ntot), part.I_Xtot)
    assert np.abs(gbn[nd]).max() == 0.0
    keys = tuple(k for k in oadj.KEYS if co.get(k) is not None)
    assert 'c12' in keys
    grads = eng.coeff_grad(ufaces, uleaf, lam, keys=keys)
    for k in keys:
        if np.abs(ref[k]).max() == 0.0:   # a coefficient that is zero everywhere has no gradient signal
            assert np.abs(grads[k].cpu().numpy()).max() == 0.0, k
            continue
        assert _rel(grads[k].cpu().numpy(), ref[k]) < 1e-9, k
    # the same gradients through the autograd function (first right-hand side)
    cs = {k: torch.as_tensor(v.ravel(), device='cuda').requires_grad_(True) for k, v in co.items() if v is not None}
    u = slab_solve(eng, torch.as_tensor(B[:, 0], device='cuda'), tol=1e-12, max_iter=40, **cs)
    (torch.as_tensor(w[:, 0], device='cuda') * u).sum().backward()
    ref1 = col.gradient(uU[:, :1], uf[:, :1], w[:, :1])
    for k in ('c12', 'c'):
        assert _rel(cs[k].grad.cpu().numpy(), ref1[k]) < 1e-9, k
    # an engine without the mixed layout has no c12 gradient
    with pytest.raises(ValueError):
        _setup(0, precision)[3].coeff_grad(ufaces, uleaf, lam, keys=('c12',))


def test_adjoint_many_right_hand_sides():
    """Columns are processed four at a time: 6 columns = 4 + 2."""
    md, part, co, eng, kh = _setup(2, 'mixed')
    rng = np.random.default_rng(11)
    nrhs = 6
    B = rng.standard_normal((md.ntot, nrhs))
    w = rng.standard_normal((md.nboxes * md.p ** 2, nrhs))
    gfv = rng.standard_normal((md.ntot, nrhs))
    col = oadj.Collocation(md, part, co)
    uU, uf, sol = col.solve(B[part.I_Xtot])
    ref = col.gradient(uU, uf, w)
    eng.factor(**_dev(co))
    uleaf, ufaces, _, _ = eng.solve(torch.as_tensor(B, device='cuda'), tol=1e-12, max_iter=40, want_faces=True)
    lam, _, gb, _, st = eng.adjoint(gleaf=torch.as_tensor(w, device='cuda'), tol=1e-12, max_iter=40)
    assert st['converged']
    lam = lam.cpu().numpy()
    for c in range(nrhs):
        assert _rel(lam[:, c], ref['lam_leaf'][:, c]) < 1e-9
        assert _rel(gb.cpu().numpy()[part.I_Xtot, c], ref['bnd'][:, c]) < 1e-9
    g = eng.coeff_grad(ufaces, uleaf, torch.as_tensor(lam, device='cuda'), keys=('c',))['c'].cpu().numpy()
    assert _rel(g, ref['c']) < 1e-9
    # a face cotangent enters the transposed system directly
    lam2, lamf2, _, _, st2 = eng.adjoint(gfaces=torch.as_tensor(gfv, device='cuda'), tol=1e-12, max_iter=40,
                                         want_faces=True)
    assert st2['converged']
    gU = np.zeros((col.nU, nrhs))
    ndf = np.flatnonzero(~col.dmask)
    gU[col.upos[ndf]] = gfv[ndf]
    lref = spsolve_t(col, gU)
    lleaf = np.zeros((md.nboxes, md.p ** 2, nrhs))
    lleaf[:, md.ld.Jc] = lref[: md.nboxes * col.n].reshape(md.nboxes, col.n, nrhs)
    assert _rel(lam2.cpu().numpy(), lleaf.reshape(-1, nrhs)) < 1e-9


def spsolve_t(col, g):
    import scipy.sparse.linalg as spla
    return spla.splu(col.K_UU.T.tocsc()).solve(g)


@pytest.mark.parametrize('precision', ['mixed', 'fp64'])
def test_autograd_gradient_matches_central_differences(precision):
    """dL/db for c = -kh^2 (1 - b(x)) through slab_solve's backward vs central differences."""
    from slablu_gb300 import slab_solve
    md, part, co, eng, kh = _setup(2, precision)
    rng = np.random.default_rng(3)
    npts = md.nboxes * md.p ** 2
    bump = torch.as_tensor(1 + co['c'].ravel() / kh ** 2, device='cuda')   # b(x) at the leaf nodes
    ones = torch.ones(npts, dtype=torch.float64, device='cuda')
    bnd = torch.as_tensor(ofuncs.uu_dir_greens(md.xx_active, kh).reshape(-1), device='cuda')
    w = torch.as_tensor(rng.standard_normal(npts), device='cuda')
    fbody = torch.as_tensor(rng.standard_normal(npts), device='cuda')

    def loss(b, bd, fb):
        u = slab_solve(eng, bd, fbody=fb, tol=1e-13, max_iter=40, c11=ones, c22=ones, c=-(kh ** 2) * (1 - b))
        return (w * u).sum()

    b = bump.clone().requires_grad_(True)
    bd = bnd.clone().requires_grad_(True)
    fb = fbody.clone().requires_grad_(True)
    L = loss(b, bd, fb)
    L.backward()
    with torch.no_grad():
        for _ in range(3):
            d = torch.as_tensor(rng.standard_normal(npts), device='cuda')
            eps = 1e-5
            fd = (loss(bump + eps * d, bnd, fbody) - loss(bump - eps * d, bnd, fbody)).item() / (2 * eps)
            ad = float((b.grad * d).sum())
            assert abs(fd - ad) <= 1e-5 * abs(fd), (fd, ad)
        # linear inputs: differences are exact up to rounding
        dd = torch.as_tensor(rng.standard_normal(bnd.shape), device='cuda')
        fd = (loss(bump, bnd + dd, fbody) - loss(bump, bnd - dd, fbody)).item() / 2
        assert abs(fd - float((bd.grad * dd).sum())) <= 1e-7 * abs(fd)
        df = torch.as_tensor(rng.standard_normal(npts), device='cuda')
        fd = (loss(bump, bnd, fbody + df) - loss(bump, bnd, fbody - df)).item() / 2
        assert abs(fd - float((fb.grad * df).sum())) <= 1e-7 * abs(fd)


def test_autograd_refuses_stale_factorization():
    from slablu_gb300 import slab_solve
    md, part, co, eng, kh = _setup(0, 'mixed')
    npts = md.nboxes * md.p ** 2
    c = torch.as_tensor(co['c'].ravel(), device='cuda').requires_grad_(True)
    ones = torch.ones(npts, dtype=torch.float64, device='cuda')
    bnd = torch.zeros(md.ntot, dtype=torch.float64, device='cuda')
    bnd[torch.as_tensor(part.I_Xtot, device='cuda')] = 1.0
    u = slab_solve(eng, bnd, c11=ones, c22=ones, c=c)
    eng.factor(c11=ones, c22=ones, c=c.detach() * 1.01)
    with pytest.raises(RuntimeError):
        u.sum().backward()


def test_config5_loss_gradient_against_dense_oracle_and_differences():
    """Config 5's inverse-scattering loss ||P u(b) - d||^2 on a reduced grid (p = 16,
    8 x 8 leaves, 4 wavelengths, the same Gaussian-random-field b, 64 seeded probes):
    dL/db from slab_solve's backward against the dense FP64 reference gradient of the
    oracle's collocation system (1e-9) and against central differences along 4 smooth
    directions (1e-5, the bench's check at full size)."""
    from slablu_gb300 import hps, problems
    from slablu_gb300.adjoint import fd_check, slab_solve
    from slablu_gb300.engine import SlabEngine
    cfg = problems.config5(n=112, nwaves=4)
    p, kh = cfg['p'], cfg['kh']
    a = cfg['a']
    geom = [[0, 1], [0, 1]]
    md = odomain.Multidomain(geom, a, p)
    part = odomain.SlabPartition(md, 1.0)
    g = hps.Geometry(geom, a, p, 1.0)
    xx = torch.as_tensor(g.xx_tot, device='cuda')
    b = cfg['b'](xx)
    ones = torch.ones_like(b)
    bnd = torch.ones(g.ntot, dtype=torch.float64, device='cuda')
    probes = torch.as_tensor(problems.probe_nodes(g.xx_tot, 64), device='cuda')
    eng = SlabEngine(g, 'fp64')
    solve = lambda bb: slab_solve(eng, bnd, tol=1e-13, max_iter=40, c11=ones, c22=ones, c=cfg['c_of_b'](bb))
    with torch.no_grad():
        d = solve(cfg['b_perturbed'](xx))[probes].clone()
    loss_fn = lambda bb: ((solve(bb)[probes] - d) ** 2).sum()
    bb = b.clone().requires_grad_(True)
    loss_fn(bb).backward()
    grad = bb.grad.detach()
    # dense FP64 reference: the oracle's collocation system with the same coefficients
    npts = g.nboxes * p * p
    co = {'c11': np.ones((g.nboxes, p * p)), 'c22': np.ones((g.nboxes, p * p)),
          'c': cfg['c_of_b'](b).cpu().numpy().reshape(g.nboxes, p * p)}
    col = oadj.Collocation(md, part, co)
    uU, uf, sol = col.solve(np.ones((part.I_Xtot.size, 1)))
    pr = probes.cpu().numpy()
    w = np.zeros((npts, 1))
    w[pr, 0] = 2 * (sol[pr, 0] - d.cpu().numpy())
    ref = col.gradient(uU, uf, w)
    ref_b = -(kh ** 2) * ref['c']
    assert _rel(grad.cpu().numpy(), ref_b) < 1e-9
    with torch.no_grad():
        for i in range(4):
            v = problems.grf(xx, seed=500 + i)
            err, h, est = fd_check(loss_fn, b, v, float((grad * v).sum()))
            assert err < 1e-5, (i, err, h, est)
