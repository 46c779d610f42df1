"""Autotuner on the GPU: candidates timed, choices applied, results unchanged."""
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


def test_tune_picks_valid_choices_and_keeps_the_solution(tmp_path):
    from slablu_gb300 import autotune, hps
    from slablu_gb300.engine import SlabEngine
    geom, p, n, kh = [[0, 1], [0, 1]], 8, 72, 45.0   # 12 x 12 leaves, 3 slabs
    a = 1 / (2 * (n / (p - 2)))
    md = odomain.Multidomain(geom, a, p)
    co = md.coeffs(ofuncs.helmholtz_pdo(lambda x: ofuncs.bfield_gaussian_bumps(x, kh)))
    coeffs = {k: torch.as_tensor(v.ravel(), device='cuda') for k, v in co.items() if v is not None}
    g = hps.Geometry(geom, a, p, 1.0)
    bnd = torch.as_tensor(np.random.default_rng(0).standard_normal(g.ntot), device='cuda')
    ref = SlabEngine(g, 'mixed')
    ref.factor(**coeffs)
    u0, _, _, _ = ref.solve(bnd, tol=1e-12, max_iter=40)
    eng = SlabEngine(g, 'mixed')
    path = str(tmp_path / 'tune.json')
    picks = autotune.tune(eng, coeffs, bnd, reps=1, path=path)
    assert picks['leaf_ctas'] in autotune.TUNABLES['leaf_ctas'][1]
    assert picks['iface_solve'] in autotune.TUNABLES['iface_solve'][1]
    assert picks['tree_tc'] in autotune.TUNABLES['tree_tc'][1]
    assert picks['gemm_tiles'] in autotune.TUNABLES['gemm_tiles'][1]
    assert eng.L.slab_engine_get_option(eng.h, autotune.TUNABLES['gemm_tiles'][0]) == picks['gemm_tiles']
    assert eng.L.slab_engine_get_option(eng.h, autotune.TUNABLES['leaf_ctas'][0]) == picks['leaf_ctas']
    u1, _, _, _ = eng.solve(bnd, tol=1e-12, max_iter=40)
    assert float(torch.linalg.norm(u1 - u0) / torch.linalg.norm(u0)) < 1e-11
    # a second engine of the same shape takes the cached choices without timing
    eng2 = SlabEngine(g, 'mixed')
    again = autotune.tune(eng2, coeffs, bnd, path=path)
    assert again['cached'] and again['leaf_ctas'] == picks['leaf_ctas']
    for key, value in ((autotune.TUNABLES['leaf_ctas'][0], 3), (autotune.TUNABLES['iface_solve'][0], 1)):
        assert eng2.L.slab_engine_set_option(eng2.h, key, value) == 0
    eng2.factor(**coeffs)
    u2, _, _, _ = eng2.solve(bnd, tol=1e-12, max_iter=40)
    assert float(torch.linalg.norm(u2 - u0) / torch.linalg.norm(u0)) < 1e-11
    assert eng2.L.slab_engine_set_option(eng2.h, 99, 0) != 0
