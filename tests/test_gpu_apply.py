"""slab_engine_apply: one application of the stored factorization to a residual.

The first refinement step of slab_engine_solve starts from the Dirichlet data
and zero unknowns, forms the FP64 residual and adds one application of the
factorization; slab_engine_residual followed by slab_engine_apply reproduces
that step, up to the order in which the application adds the two leaves'
fluxes to each face row (atomics: 1e-12 relative with FP64 factors, 1e-4 with
FP32 factors, where the measured spread between runs is 2e-6).  Dirichlet
entries of the face residual are ignored and the correction is zero there, and
the step reduces the FP64 residual by orders of magnitude.  In FP64 one
application is already the solution to 1e-9 against the oracle's sparse direct
solve (the engine's solve is held to the oracle by test_gpu_parity.py).
"""
import numpy as np
import pytest
import torch

from oracle import adjoint as oadj
from oracle import domain as odomain
from oracle import funcs as ofuncs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.fail('GPU tests need CUDA')
    from slablu_gb300 import build
    build.build()


def _rel(x, y):
    return float(torch.linalg.norm(x - y) / torch.linalg.norm(y))


@pytest.mark.parametrize('precision', ['fp64', 'fp32'])
def test_apply_is_one_refinement_step(precision):
    from slablu_gb300 import hps
    from slablu_gb300.engine import SlabEngine
    geom, p, n, kh = [[0, 1], [0, 1]], 8, 48, 30.0
    a = 1 / (2 * (n / (p - 2)))
    md = odomain.Multidomain(geom, a, p)
    part = odomain.SlabPartition(md, 1.0)
    co = md.coeffs(ofuncs.helmholtz_pdo(lambda x: ofuncs.bfield_gaussian_bumps(x, kh)))
    g = hps.Geometry(geom, a, p, 1.0)
    eng = SlabEngine(g, precision)
    eng.factor(**{k: torch.as_tensor(v.ravel(), device='cuda') for k, v in co.items() if v is not None})
    nrhs = 2
    gen = torch.Generator(device='cuda').manual_seed(5)
    bnd = torch.randn(g.ntot, nrhs, generator=gen, device='cuda', dtype=torch.float64)
    dirm = torch.zeros(g.ntot, dtype=torch.bool, device='cuda')
    dirm[torch.as_tensor(g.I_Xtot, device='cuda')] = True
    bnd = bnd.masked_fill(~dirm[:, None], 0.0)            # data on the Dirichlet faces only
    uleaf1, uf1, it, _ = eng.solve(bnd, tol=0.0, max_iter=1, want_faces=True, allow_noconv=True)
    assert it == 1
    q = p - 2
    r = torch.arange(q * q, device='cuda')
    node = (r // q + 1) * p + (r % q + 1)
    uint0 = torch.zeros(eng.nleaf, nrhs, q * q, dtype=torch.float64, device='cuda')
    rint, rf = eng.residual(bnd, uint0)
    # Dirichlet entries of the face residual are not read
    rf_noise = rf + torch.randn(rf.shape, generator=gen, device='cuda', dtype=torch.float64) * dirm[:, None]
    dint, df = eng.apply(rint, rf_noise)
    assert float(df[dirm].abs().max()) == 0.0
    tol = 1e-12 if precision == 'fp64' else 1e-4
    assert _rel(bnd + df, uf1) < tol
    ref_int = uleaf1.T.reshape(nrhs, eng.nleaf, p * p)[:, :, node].permute(1, 0, 2)
    assert _rel(dint, ref_int) < tol
    r1i, r1f = eng.residual(bnd + df, dint)
    r0n = float(torch.sqrt(torch.sum(rint ** 2) + torch.sum(rf ** 2)))
    r1n = float(torch.sqrt(torch.sum(r1i ** 2) + torch.sum(r1f ** 2)))
    assert r1n < (1e-9 if precision == 'fp64' else 1e-3) * r0n, (r1n, r0n)
    if precision == 'fp64':
        col = oadj.Collocation(md, part, co)
        _, uf_ref, _ = col.solve(bnd.cpu().numpy()[part.I_Xtot])
        e = np.linalg.norm((bnd + df).cpu().numpy() - uf_ref) / np.linalg.norm(uf_ref)
        assert e < 1e-9, e
    with pytest.raises(ValueError):
        eng.apply(rint[:, :1, :-1], rf)
