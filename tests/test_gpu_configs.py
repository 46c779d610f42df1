"""The benchmark configurations on the GPU against the reference's own runs.

Fixtures (tests/golden/make_golden.py, which runs the unmodified reference):
  config 1  p = 12, n = 400, 8 seeded plane waves: the reference's slabLU solution;
  config 2  16,384 leaves of a 128 x 128 tiling, p = 22, 32-bump field: the
            reference's form_DtNs on a sample of the leaves;
  config 3  p = 22, n = 2000 (N = 4,404,000), Gaussian lattice, u = 1: the
            reference's slabLU solution (and two of config 4's right-hand sides
            on the same factorization).
The headline metric asks for at most 1e-6 relative error against the FP64
oracle; the tests hold every precision mode to that bar at full size, and the
FP64 leaf maps to 1e-10.
"""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), 'golden')
TOL_METRIC = 1e-6     # relative error bar of the headline metric


@pytest.fixture(scope='module', autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.fail('GPU tests need CUDA')
    from slablu_gb300 import build
    build.build()


def _solver(cfg, precision, tol=1e-10):
    import slablu_gb300 as sg
    op = sg.pdo.PDO_2d(sg.pdo.ones, sg.pdo.ones, c=cfg['c'])
    dom = sg.Domain_Solver(torch.tensor([[0, 1.0], [0, 1.0]]), op, cfg['kh'], cfg['a'], p=cfg['p'],
                           buf_constant=1.0, precision=precision, tol=tol)
    dom.build('reduced_gpu', 'slabLU', verbose=False)
    return dom


def _rel(sol, g, key='sol'):
    stride = int(g['stride'])
    ref = g[key + '_sub']
    return float(np.linalg.norm(sol[::stride] - ref) / np.linalg.norm(ref))


@pytest.mark.parametrize('precision', ['fp64', 'mixed', 'fp32'])
def test_config1_plane_waves(precision):
    from slablu_gb300 import problems
    g = np.load(os.path.join(GOLD, 'config1_slabLU_p12_n400.npz'))
    cfg = problems.config1()
    dom = _solver(cfg, precision)
    sol, rel, _, _, _ = dom.solve(cfg['uu_dir'], None)
    sol = sol.numpy()[:, 0]
    assert sol.size == int(g['sol_len'])
    assert _rel(sol, g) < 1e-8
    assert abs(np.linalg.norm(sol) - float(g['sol_norm'])) < 1e-8 * float(g['sol_norm'])
    assert float(rel) < 1e-10


def test_config2_leaf_dtn_against_reference():
    """FP64 leaf maps to 1e-10 of the reference's, FP32 maps to 2e-4, on the sampled leaves."""
    from slablu_gb300 import hps, leaf_dtn
    g = np.load(os.path.join(GOLD, 'config2_dtn_p22.npz'))
    p = int(g['p'])
    ops = hps.LeafOps(float(g['a']), p)
    n = g['c'].shape[0]
    co = {'c11': torch.ones(n, p * p, dtype=torch.float64, device='cuda'),
          'c22': torch.ones(n, p * p, dtype=torch.float64, device='cuda'),
          'c': torch.as_tensor(g['c'], device='cuda')}
    ref = g['dtn']
    for prec, tol in (('fp64', 1e-10), ('fp32', 2e-4)):
        dtn, info = leaf_dtn(co, p, ops.D, ops.Dsq, ops.Nx, precision=prec)
        assert int(info.abs().sum()) == 0
        rel = np.linalg.norm(dtn.cpu().numpy() - ref, axis=(1, 2)) / np.linalg.norm(ref, axis=(1, 2))
        assert rel.max() < tol, (prec, rel.max())


def test_config2_all_leaves_fp32_against_fp64():
    """All 16,384 leaves: per-leaf relative error of the FP32 maps against the FP64 maps.
    Most leaves agree to ~1e-6 (median below 1e-5); leaves whose interior block is
    close to a Helmholtz resonance (kh = 1610 here) amplify the FP32 rounding by
    their condition number (a few percent at worst), which is why the FP32 factors
    are only a preconditioner and the solution is refined against the FP64 residual."""
    from slablu_gb300 import hps, leaf_dtn, problems
    cfg = problems.config2()
    p = cfg['p']
    geo = hps.Geometry([[0, 1], [0, 1]], cfg['a'], p, 1.0)
    xx = torch.as_tensor(geo.xx_tot, device='cuda')
    nl = geo.nboxes
    assert nl == 16384
    co = {'c11': torch.ones(nl, p * p, dtype=torch.float64, device='cuda'),
          'c22': torch.ones(nl, p * p, dtype=torch.float64, device='cuda'),
          'c': cfg['c'](xx).reshape(nl, p * p).contiguous()}
    d64, i64 = leaf_dtn(co, p, geo.ops.D, geo.ops.Dsq, geo.ops.Nx, precision='fp64')
    d32, i32 = leaf_dtn(co, p, geo.ops.D, geo.ops.Dsq, geo.ops.Nx, precision='fp32')
    assert int(i64.abs().sum()) == 0 and int(i32.abs().sum()) == 0
    rel = torch.linalg.norm((d32 - d64).flatten(1), dim=1) / torch.linalg.norm(d64.flatten(1), dim=1)
    assert torch.isfinite(rel).all()
    assert float(rel.median()) < 1e-5, float(rel.median())
    assert float(rel.max()) < 0.2, float(rel.max())


@pytest.fixture(scope='module')
def config3_mixed():
    from slablu_gb300 import problems
    cfg = problems.config3()
    return cfg, _solver(cfg, 'mixed', tol=1e-6)


@pytest.fixture(scope='module')
def config3_fp32():
    from slablu_gb300 import problems
    cfg = problems.config3()
    return cfg, _solver(cfg, 'fp32', tol=1e-6)


@pytest.mark.parametrize('precision', ['fp32', 'mixed'])
@pytest.mark.parametrize('solver', ['superLU', 'slabLU'])
def test_config3_reduced_precision_against_reference(request, precision, solver):
    """The benchmark's workload and refinement tolerance (1e-6 on the relative
    correction), with every factor in FP32 (the benchmark's mode) and with the
    FP64 interface factorization: the leaf-node solution within the metric's 1e-6
    of the reference's FP64 solutions at N = 4,404,000 (its superLU sparse direct
    solve and its slabLU, which differ from each other by 4e-8)."""
    cfg, dom = request.getfixturevalue(f'config3_{precision}')
    g = np.load(os.path.join(GOLD, f'config3_{solver}_p22_n2000.npz'))
    sol, rel, _, _, _ = dom.solve(cfg['uu_dir'], None)
    sol = sol.numpy()[:, 0]
    assert sol.size == int(g['sol_len'])
    err = _rel(sol, g)
    assert err < TOL_METRIC, err
    assert abs(np.linalg.norm(sol) - float(g['sol_norm'])) < TOL_METRIC * float(g['sol_norm'])


def test_config3_fp64_against_superlu():
    """The plain all-FP64 GPU path at N = 4,404,000 against the reference's superLU solution."""
    from slablu_gb300 import problems
    cfg = problems.config3()
    dom = _solver(cfg, 'fp64', tol=1e-10)
    g = np.load(os.path.join(GOLD, 'config3_superLU_p22_n2000.npz'))
    sol, rel, _, _, _ = dom.solve(cfg['uu_dir'], None)
    err = _rel(sol.numpy()[:, 0], g)
    assert err < 1e-7, err
    del dom
    torch.cuda.empty_cache()


def test_config4_columns_against_reference(config3_fp32):
    """Config 4's smoothed random boundary data (columns 0 and 255 of the 256) on the
    config-3 factorization (FP32 factors, as in the benchmark), solved together,
    against the reference's solutions."""
    from slablu_gb300 import problems
    cfg, dom = config3_fp32
    g = np.load(os.path.join(GOLD, 'config3_slabLU_p22_n2000.npz'))
    B = problems.config4_rhs(int(g['nbnd']), 256)
    cols = [int(c) for c in g['rhs_cols']]
    data = B[:, cols]

    def uu(xx):
        assert xx.shape[0] == data.shape[0]
        return data
    sol, _, _, _, _ = dom.solve(uu, None)
    sol = sol.numpy()
    for k in range(len(cols)):
        err = _rel(sol[:, k], g, f'rhs{k}_sol')
        assert err < TOL_METRIC, (cols[k], err)
