"""The refined solves of several engines as one CUDA graph (slab_solve_graph_*).

The graph runs the same kernels in the same order as slab_engine_solve, with
the refinement decision taken on the device, so its solutions match
slab_engine_solve's to rounding (1e-13 relative measured; 1e-11 asserted, and
the step counts within one, because the FP32 face sums of an application are
atomic and their order can change the last bits of a step); slab_engine_solve
is itself held to the oracle by test_gpu_parity.py.  Also: a second launch with new inputs, a re-factorization
picked up without a new graph, and the host-side refusals (an engine given
twice; buffers reallocated after the graph was made).
"""
import numpy as np
import pytest
import torch

from oracle import domain as odomain
from oracle import funcs as ofuncs

pytestmark = pytest.mark.gpu

# (box, p, n, kh, precision, nrhs, body load)
CASES = [
    ([[0, 1], [0, 1]], 8, 48, 30.0, 'mixed', 1, False),
    ([[0, 1], [0, 1]], 22, 80, 30.0, 'mixed', 3, True),
    ([[0, 1], [0, 0.5]], 12, 60, 20.0, 'fp64', 2, False),
]


@pytest.fixture(scope='module', autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.fail('GPU tests need CUDA')
    from slablu_gb300 import build
    build.build()


def _engine(case, kh_scale=1.0):
    from slablu_gb300 import hps
    from slablu_gb300.engine import SlabEngine
    geom, p, n, kh, prec, _, _ = CASES[case]
    a = 1 / (2 * (n / (p - 2)))
    md = odomain.Multidomain(geom, a, p)
    co = md.coeffs(ofuncs.helmholtz_pdo(lambda x: ofuncs.bfield_gaussian_bumps(x, kh * kh_scale)))
    eng = SlabEngine(hps.Geometry(geom, a, p, 1.0), prec)
    eng.factor(**{k: torch.as_tensor(v.ravel(), device='cuda') for k, v in co.items() if v is not None})
    return eng


def _inputs(eng, case, seed):
    nrhs, body = CASES[case][5], CASES[case][6]
    gen = torch.Generator(device='cuda').manual_seed(seed)
    bnd = torch.randn(eng.ntot, nrhs, generator=gen, device='cuda', dtype=torch.float64)
    fb = torch.randn(eng.npts, nrhs, generator=gen, device='cuda', dtype=torch.float64) if body else None
    return bnd, fb


def _rel(x, y):
    return float(torch.linalg.norm(x - y) / torch.linalg.norm(y))


TOL, MAXIT = 1e-12, 40


def _check(graph, engines, inputs):
    graph.launch()
    for i, (eng, (bnd, fb)) in enumerate(zip(engines, inputs)):
        u_ref, _, it_ref, info_ref = eng.solve(bnd, fb, tol=TOL, max_iter=MAXIT)
        u, it, info = graph.result(i)
        assert info['converged']
        assert abs(it - it_ref) <= 1, (i, it, it_ref)
        assert _rel(u, u_ref) < 1e-11, (i, _rel(u, u_ref))
        assert info['rel_correction'] <= TOL
        assert abs(info['residual'] - info_ref['residual']) <= 1e-6 * info_ref['residual0']


def test_solve_graph_matches_engine_solve():
    from slablu_gb300 import SolveGraph
    engines = [_engine(c) for c in range(len(CASES))]
    graph = SolveGraph(engines, nrhs=[c[5] for c in CASES], with_fbody=True, tol=TOL, max_iter=MAXIT)
    for seed in (1, 2):  # two launches with new inputs
        inputs = [_inputs(e, c, seed * 10 + c) for c, e in enumerate(engines)]
        for i, (bnd, fb) in enumerate(inputs):
            graph.set_inputs(i, bnd, fb)
        _check(graph, engines, inputs)
    # new coefficients (same set): the graph solves with the new factors
    fresh = _engine(0, kh_scale=1.3)
    co_state = fresh._coef
    engines[0].factor(*co_state[:5])
    _check(graph, engines, inputs)


def test_solve_graph_refusals():
    from slablu_gb300 import SolveGraph, _lib
    eng = _engine(0)
    with pytest.raises(_lib.SlabError):
        SolveGraph([eng, eng], nrhs=1)
    graph = SolveGraph([eng], nrhs=1, tol=TOL, max_iter=MAXIT)
    bnd, _ = _inputs(eng, 0, 5)
    graph.set_inputs(0, bnd)
    graph.launch()
    graph.result(0)
    eng.solve(torch.cat([bnd] * 5, dim=1), tol=TOL, max_iter=MAXIT)  # grows the solve buffers
    with pytest.raises(_lib.SlabError) as ex:
        graph.launch()
    assert ex.value.status == -4
    np.testing.assert_equal(SolveGraph([eng], nrhs=1).nrhs, [1])


def test_solve_graph_with_mixed_derivative_engine():
    """An engine with c12 (curvy-annulus coefficients, 8 x 8 leaves of order 8) next to
    one without, in one graph: the same steps and solutions as slab_engine_solve."""
    from slablu_gb300 import SolveGraph, hps
    from slablu_gb300.engine import SlabEngine
    p, n, kh = 8, 48, 12.0
    a = 1 / (2 * (n / (p - 2)))
    md = odomain.Multidomain([[0, 1], [0, 1]], a, p)
    g = hps.Geometry([[0, 1], [0, 1]], a, p, 1.0)
    pdo, _ = ofuncs.curvy_annulus_pdo(kh, ofuncs.bfield_constant)
    co = md.coeffs(pdo)
    emix = SlabEngine(g, 'mixed', mixed=True)
    emix.factor(**{k: torch.as_tensor(v.ravel(), device='cuda') for k, v in co.items() if v is not None})
    engines = [emix, _engine(0)]
    graph = SolveGraph(engines, nrhs=[2, 1], tol=TOL, max_iter=MAXIT)
    gen = torch.Generator(device='cuda').manual_seed(9)
    inputs = [(torch.randn(e.ntot, k, generator=gen, device='cuda', dtype=torch.float64), None)
              for e, k in zip(engines, (2, 1))]
    for i, (bnd, fb) in enumerate(inputs):
        graph.set_inputs(i, bnd, fb)
    _check(graph, engines, inputs)
