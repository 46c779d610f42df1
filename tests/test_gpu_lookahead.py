"""Interface block LU with lookahead (second stream) against the serial order.

The lookahead moves each outer block's update of the far columns to a second
stream and applies the panels' row interchanges to those columns later, as
one gather; the arithmetic is unchanged, so both orders give the same
factors and, after refinement, the same solution.  The interface block here has 520 unknowns (130 leaves of p = 6 per
slab interface), so the first outer block forks work to the second stream.
"""
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


def test_lookahead_matches_serial_order_and_oracle():
    from slablu_gb300 import _lib, hps
    from slablu_gb300.engine import SlabEngine
    p, kh, n1 = 6, 20.0, 130
    a = 1 / (2 * n1)
    geom = [[0, 4 * 2 * a], [0, 1]]  # 4 x 130 leaves
    md = odomain.Multidomain(geom, a, p)
    part = odomain.SlabPartition(md, 0.05)
    co = md.coeffs(ofuncs.helmholtz_pdo(lambda x: ofuncs.bfield_gaussian_bumps(x, kh)))
    ud = lambda x: ofuncs.uu_dir_greens(x, kh)
    ref = odomain.solve_full(md, part, co, ud)['sol_tot'][:, 0]
    g = hps.Geometry(geom, a, p, 0.05)
    assert g.Npan == 2 and g.n1 * g.q > 2 * 256
    coeffs = {k: torch.as_tensor(v.ravel(), device='cuda') for k, v in co.items() if v is not None}
    bnd = torch.as_tensor(ud(md.xx_active), device='cuda')
    sols = {}
    for la in (0, 1):
        eng = SlabEngine(g, 'mixed')
        assert eng.L.slab_engine_set_option(eng.h, _lib.SLAB_OPT_IFACE_LOOKAHEAD, la) == 0
        assert eng.L.slab_engine_get_option(eng.h, _lib.SLAB_OPT_IFACE_LOOKAHEAD) == la
        eng.factor(**coeffs)
        u, _, iters, st = eng.solve(bnd, tol=1e-12, max_iter=40)
        assert st['converged'], (la, iters, st)
        sols[la] = u[:, 0].cpu().numpy()
    # both are refined to a relative correction of 1e-12; the split-k products of
    # the solve accumulate with atomics, so the two runs agree to the refinement
    # level, not bit for bit
    diff = np.linalg.norm(sols[1] - sols[0]) / np.linalg.norm(sols[0])
    assert diff < 1e-11, diff
    rel = np.linalg.norm(sols[1] - ref) / np.linalg.norm(ref)
    assert rel < 1e-9, rel


@pytest.mark.parametrize('nblocks', [3, 4])
def test_outer_inverse_schur_solves_match_fp64_core_solves_and_oracle(nblocks):
    """The Schur right-hand sides X_j = S_j^{-1} sup_j through inverted 256-row
    diagonal blocks of L and U (every product on the tensor cores,
    SLAB_OPT_IFACE_OUTER_INV = 1) against the FP64-core triangular solves of 64-row
    blocks (0): same solution after refinement, and the oracle's.  Interface blocks
    of 520 unknowns: two full 256-row outer blocks and a partial one of 8 rows."""
    from slablu_gb300 import _lib, hps
    from slablu_gb300.engine import SlabEngine
    p, kh, n1 = 6, 20.0, 130
    a = 1 / (2 * n1)
    geom = [[0, 2 * nblocks * 2 * a], [0, 1]]  # 2 leaf columns per slab
    md = odomain.Multidomain(geom, a, p)
    part = odomain.SlabPartition(md, 0.05)
    co = md.coeffs(ofuncs.helmholtz_pdo(lambda x: ofuncs.bfield_gaussian_bumps(x, kh)))
    ud = lambda x: ofuncs.uu_dir_greens(x, kh)
    ref = odomain.solve_full(md, part, co, ud)['sol_tot'][:, 0]
    g = hps.Geometry(geom, a, p, 0.05)
    assert g.Npan >= 3 and g.n1 * g.q > 2 * 256
    coeffs = {k: torch.as_tensor(v.ravel(), device='cuda') for k, v in co.items() if v is not None}
    bnd = torch.as_tensor(ud(md.xx_active), device='cuda')
    sols = {}
    for oi in (0, 1):
        eng = SlabEngine(g, 'mixed')
        assert eng.L.slab_engine_set_option(eng.h, _lib.SLAB_OPT_IFACE_OUTER_INV, oi) == 0
        assert eng.L.slab_engine_get_option(eng.h, _lib.SLAB_OPT_IFACE_OUTER_INV) == oi
        eng.factor(**coeffs)
        u, _, iters, st = eng.solve(bnd, tol=1e-12, max_iter=40)
        assert st['converged'], (oi, iters, st)
        sols[oi] = u[:, 0].cpu().numpy()
    diff = np.linalg.norm(sols[1] - sols[0]) / np.linalg.norm(sols[0])
    assert diff < 1e-11, diff
    rel = np.linalg.norm(sols[1] - ref) / np.linalg.norm(ref)
    assert rel < 1e-9, rel


def test_fp32_panel_in_one_cta_matches_cluster_panel():
    """FP32 interface panels factored in one CTA (SLAB_OPT_IFACE_PANEL 0) against
    the thread-block-cluster kernel (1): the same pivot sequence and operations,
    so the same factors.  Interface blocks of 2,080 unknowns (520 leaves of p = 6
    per slab interface, two interfaces): the first panels are taller than the
    one-CTA kernel takes (1,536 rows) and go to the cluster kernel, the rest use
    512 threads with shared-memory rows (above 1,024 rows), 512, 256 and 128
    threads with register rows only."""
    from slablu_gb300 import _lib, hps
    from slablu_gb300.engine import SlabEngine
    p, kh, n1 = 6, 20.0, 520
    a = 1 / (2 * n1)
    geom = [[0, 6 * 2 * a], [0, 1]]  # 6 x 520 leaves, three slabs of two leaf columns
    g = hps.Geometry(geom, a, p, 0.02)
    assert g.Npan == 3 and g.n1 * g.q == 2080
    xx = torch.as_tensor(g.xx_tot, device='cuda')
    c = (-kh ** 2 * (1 - 0.5 * torch.exp(-((xx[:, 0] - 0.01) ** 2 + (xx[:, 1] - 0.5) ** 2) / 0.02))).contiguous()
    one = torch.ones_like(c)
    gen = torch.Generator(device='cuda').manual_seed(3)
    bnd = torch.randn(g.ntot, 2, generator=gen, device='cuda', dtype=torch.float64)
    sols = {}
    for kind in (1, 0):
        eng = SlabEngine(g, 'fp32')
        assert eng.L.slab_engine_set_option(eng.h, _lib.SLAB_OPT_IFACE_PANEL, kind) == 0
        assert eng.L.slab_engine_get_option(eng.h, _lib.SLAB_OPT_IFACE_PANEL) == kind
        eng.factor(c11=one, c22=one, c=c)
        u, _, iters, st = eng.solve(bnd, tol=1e-12, max_iter=60)
        assert st['converged'], (kind, iters, st)
        sols[kind] = (u.cpu().numpy(), iters)
    e64 = SlabEngine(g, 'fp64')
    e64.factor(c11=one, c22=one, c=c)
    u64 = e64.solve(bnd, tol=1e-13, max_iter=10)[0].cpu().numpy()
    assert sols[0][1] == sols[1][1]
    diff = np.linalg.norm(sols[0][0] - sols[1][0]) / np.linalg.norm(sols[1][0])
    assert diff < 1e-11, diff
    for kind in (0, 1):
        rel = np.linalg.norm(sols[kind][0] - u64) / np.linalg.norm(u64)
        assert rel < 1e-9, (kind, rel)


def test_fp32_blocked_interface_lu_matches_unblocked(monkeypatch):
    """FP32 interface blocks factored in 256-column outer blocks (biglu_blocked),
    with and without the lookahead stream, against the unblocked panel-by-panel
    LU: the same elimination with the products grouped differently, so after
    refinement the solutions agree to the refinement level.  Interface blocks
    of 2,080 unknowns (nine outer blocks each)."""
    from slablu_gb300 import _lib, hps
    from slablu_gb300.engine import SlabEngine
    p, kh, n1 = 6, 20.0, 520
    a = 1 / (2 * n1)
    g = hps.Geometry([[0, 6 * 2 * a], [0, 1]], a, p, 0.02)
    assert g.Npan == 3
    xx = torch.as_tensor(g.xx_tot, device='cuda')
    c = (-kh ** 2 * (1 - 0.5 * torch.exp(-((xx[:, 0] - 0.01) ** 2 + (xx[:, 1] - 0.5) ** 2) / 0.02))).contiguous()
    one = torch.ones_like(c)
    gen = torch.Generator(device='cuda').manual_seed(4)
    bnd = torch.randn(g.ntot, 1, generator=gen, device='cuda', dtype=torch.float64)
    sols = {}
    for name, unblocked, la in (('unblocked', '1', 1), ('serial', '0', 0), ('lookahead', '0', 1)):
        monkeypatch.setenv('SLAB_IFACE_UNBLOCKED', unblocked)
        eng = SlabEngine(g, 'fp32')
        assert eng.L.slab_engine_set_option(eng.h, _lib.SLAB_OPT_IFACE_LOOKAHEAD, la) == 0
        eng.factor(c11=one, c22=one, c=c)
        u, _, iters, st = eng.solve(bnd, tol=1e-12, max_iter=60)
        assert st['converged'], (name, iters, st)
        sols[name] = (u[:, 0].cpu().numpy(), iters)
    ref, it_ref = sols['unblocked']
    for name in ('serial', 'lookahead'):
        u, it = sols[name]
        assert abs(it - it_ref) <= 1, (name, it, it_ref)
        diff = np.linalg.norm(u - ref) / np.linalg.norm(ref)
        assert diff < 1e-11, (name, diff)
    assert np.array_equal(sols['serial'][0], sols['lookahead'][0]) or \
        np.linalg.norm(sols['serial'][0] - sols['lookahead'][0]) < 1e-11 * np.linalg.norm(ref)


def test_fp32_products_on_128_tiles_match_64_tiles(monkeypatch):
    """The FP32 products with both sides at least 128 run on 128 x 128 tiles
    (gemm128_kernel); SLAB_GEMM64=1, or the engine option SLAB_OPT_GEMM_TILES =
    1, keeps them on the 64 x 64 kernel.  Both sum each entry's k terms in the
    same order; the refined solutions agree with each other and with the FP64
    engine to the refinement level (interface blocks of 2,080, merge fronts up
    to 1,040)."""
    from slablu_gb300 import hps
    from slablu_gb300.engine import SlabEngine
    p, kh, n1 = 6, 20.0, 520
    a = 1 / (2 * n1)
    g = hps.Geometry([[0, 6 * 2 * a], [0, 1]], a, p, 0.02)
    xx = torch.as_tensor(g.xx_tot, device='cuda')
    c = (-kh ** 2 * (1 - 0.5 * torch.exp(-((xx[:, 0] - 0.01) ** 2 + (xx[:, 1] - 0.5) ** 2) / 0.02))).contiguous()
    one = torch.ones_like(c)
    gen = torch.Generator(device='cuda').manual_seed(5)
    bnd = torch.randn(g.ntot, 2, generator=gen, device='cuda', dtype=torch.float64)
    from slablu_gb300 import _lib
    sols = {}
    for flag in ('1', '0'):
        monkeypatch.setenv('SLAB_GEMM64', flag)
        for prec in ('fp32', 'mixed'):
            eng = SlabEngine(g, prec)
            eng.factor(c11=one, c22=one, c=c)
            u, _, iters, st = eng.solve(bnd, tol=1e-12, max_iter=60)
            assert st['converged'], (flag, prec, iters, st)
            sols[flag, prec] = u.cpu().numpy()
    monkeypatch.setenv('SLAB_GEMM64', '0')
    for prec in ('fp32', 'mixed'):  # the same 64 x 64 choice as an engine option
        eng = SlabEngine(g, prec)
        assert eng.L.slab_engine_set_option(eng.h, _lib.SLAB_OPT_GEMM_TILES, 1) == 0
        assert eng.L.slab_engine_get_option(eng.h, _lib.SLAB_OPT_GEMM_TILES) == 1
        eng.factor(c11=one, c22=one, c=c)
        u, _, iters, st = eng.solve(bnd, tol=1e-12, max_iter=60)
        assert st['converged'], ('option', prec, iters, st)
        assert np.array_equal(u.cpu().numpy(), sols['1', prec]) or \
            np.linalg.norm(u.cpu().numpy() - sols['1', prec]) < 1e-11 * np.linalg.norm(sols['1', prec])
    e64 = SlabEngine(g, 'fp64')
    e64.factor(c11=one, c22=one, c=c)
    u64 = e64.solve(bnd, tol=1e-13, max_iter=10)[0].cpu().numpy()
    for key, u in sols.items():
        rel = np.linalg.norm(u - u64) / np.linalg.norm(u64)
        assert rel < 1e-9, (key, rel)
