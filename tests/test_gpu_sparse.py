"""Reduced sparse operator on the GPU against the oracle's SciPy assembly.

Tolerances: the device sum of the same FP64 DtN values is bit-exact (at most two
terms meet in a slot); with the GPU's own FP64 leaf DtN maps the operator agrees
to 1e-10 relative, as the DtN maps do.
"""
import numpy as np
import pytest
import torch

from oracle import domain as odomain
from oracle import funcs as ofuncs
from oracle import leaf as oleaf

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.fail('GPU tests need CUDA')
    from slablu_gb300 import build
    build.build()


def _problem(geom=((0, 1), (0, 1)), p=8, n=48, kh=30.0):
    a = 1 / (2 * (n / (p - 2)))
    md = odomain.Multidomain(geom, a, p)
    part = odomain.SlabPartition(md, 1.0)
    co = md.coeffs(ofuncs.helmholtz_pdo(lambda x: ofuncs.bfield_gaussian_bumps(x, kh)))
    return a, md, part, co, kh


def test_csr_assembly_of_oracle_dtns_is_exact():
    from slablu_gb300 import hps, sparse
    a, md, part, co, _ = _problem()
    dtn = oleaf.dtn_build(md.ld, co)
    ref = md.sparse_mat(dtn)
    ref.sort_indices()
    g = hps.Geometry([[0, 1], [0, 1]], a, md.p, 1.0)
    A = sparse.assemble(g, torch.as_tensor(dtn, device='cuda'))
    assert np.array_equal(A.indptr.cpu().numpy(), ref.indptr)
    assert np.array_equal(A.indices.cpu().numpy(), ref.indices)
    assert np.array_equal(A.vals.cpu().numpy(), ref.data)
    # product, one and three columns
    rng = np.random.default_rng(1)
    for k in (1, 3):
        x = rng.standard_normal((md.ntot, k)) if k > 1 else rng.standard_normal(md.ntot)
        y = A.matvec(torch.as_tensor(x, device='cuda')).cpu().numpy()
        yr = ref @ x
        assert np.linalg.norm(y - yr) <= 1e-14 * np.linalg.norm(yr)
    y0 = torch.as_tensor(rng.standard_normal(md.ntot), device='cuda')
    x = torch.as_tensor(rng.standard_normal(md.ntot), device='cuda')
    y = A.matvec(x, alpha=2.0, beta=-0.5, y=y0.clone()).cpu().numpy()
    yr = 2.0 * (ref @ x.cpu().numpy()) - 0.5 * y0.cpu().numpy()
    assert np.linalg.norm(y - yr) <= 1e-14 * np.linalg.norm(yr)


def test_domain_solver_sparse_mat_and_rhs_match_oracle():
    import slablu_gb300 as sg
    a, md, part, co, kh = _problem()
    op = sg.pdo.PDO_2d(sg.pdo.ones, sg.pdo.ones, c=lambda xx: sg.built_in_funcs.bfield_gaussian_bumps(xx, kh))
    dom = sg.Domain_Solver(torch.tensor([[0, 1.], [0, 1.]]), op, kh, a, p=md.p, buf_constant=1.0)
    A, t = dom.hps.sparse_mat('cuda')
    assert A.layout == torch.sparse_csr and set(t) >= {'toc_DtN', 'toc_sparse'}
    ref = md.sparse_mat(oleaf.dtn_build(md.ld, co))
    ref.sort_indices()
    vals = A.values().cpu().numpy()
    assert np.array_equal(A.crow_indices().cpu().numpy(), ref.indptr)
    assert np.linalg.norm(vals - ref.data) <= 1e-10 * np.linalg.norm(ref.data)
    ud = lambda x: ofuncs.uu_dir_greens(np.asarray(x), kh)
    ff = dom.get_rhs(lambda xx: torch.as_tensor(ud(xx)))
    ffr = odomain.dirichlet_rhs(ref, part, ud(md.xx_active[part.I_Xtot]))
    ffr = ffr.reshape(ff.shape)
    assert np.linalg.norm(ff.cpu().numpy() - ffr) <= 1e-10 * np.linalg.norm(ffr)
