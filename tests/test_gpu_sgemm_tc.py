"""FP32 GEMM on the TF32 tensor cores (three-way split) against an FP64 product.

The split is exact and the six slice products cover every weight down to
2^-22, so what is left is the FP32 accumulation in tensor memory: the tests
bound the error per entry by 4 k 2^-24 max|A(i,:)| max|B(:,j)| (the FP32
worst-case dot-product bound with a 4x margin) and normwise by 1e-5 (measured
1.5e-6 at k = 200, ~25 FP32 units: the tensor core's accumulation rounds less
tightly than a chain of FMAs; a single TF32 product would give ~1e-3).
"""
import pytest
import torch

pytestmark = pytest.mark.gpu

F32 = torch.float32   # the package sets the default dtype to float64, as the reference does


@pytest.fixture(scope='module', autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.fail('GPU tests need CUDA')
    from slablu_gb300 import build
    build.build()


def _check(A, B, C=None, alpha=1.0, beta=0.0):
    from slablu_gb300.dgemm import sgemm_tc
    A64, B64 = A.double(), B.double()
    ref = alpha * (A64 @ B64) + (beta * C.double() if C is not None else 0.0)
    out = sgemm_tc(A, B, None if C is None else C.clone(), alpha=alpha, beta=beta).double()
    k = A.shape[-1]
    scale = A64.abs().amax(dim=-1, keepdim=True) * B64.abs().amax(dim=-2, keepdim=True) * abs(alpha)
    if C is not None:
        scale = scale + abs(beta) * C.double().abs()
    err = ((out - ref).abs() / (scale + 1e-30)).max().item()
    assert err <= 4 * k * 2.0 ** -24, err
    return out, ref


@pytest.mark.parametrize('b,m,n,k', [(1, 1, 1, 1), (1, 128, 128, 32), (3, 200, 1000, 200), (2, 130, 70, 33),
                                     (5, 64, 40, 7), (1, 1000, 2000, 200), (2, 4000, 300, 200)])
def test_sgemm_tc_random(b, m, n, k):
    g = torch.Generator(device='cuda').manual_seed(b * 1000 + m + n + k)
    A = torch.randn(b, m, k, device='cuda', generator=g, dtype=F32)
    B = torch.randn(b, k, n, device='cuda', generator=g, dtype=F32)
    out, ref = _check(A, B)
    rel = (torch.linalg.norm(out - ref) / torch.linalg.norm(ref)).item()
    assert rel < 1e-5, rel


def test_sgemm_tc_scaled_and_beta():
    g = torch.Generator(device='cuda').manual_seed(3)
    m, n, k = 300, 96, 250
    A = torch.randn(m, k, device='cuda', generator=g, dtype=F32) * torch.logspace(-10, 10, m, device='cuda', dtype=F32)[:, None]
    B = torch.randn(k, n, device='cuda', generator=g, dtype=F32) * torch.logspace(8, -8, n, device='cuda', dtype=F32)[None, :]
    C = torch.randn(m, n, device='cuda', generator=g, dtype=F32)
    _check(A, B, C, alpha=-1.0, beta=1.0)


def test_sgemm_tc_output_aliases_b():
    """C may be B itself (the slab merges form W = M^{-1} R in place of R)."""
    from slablu_gb300 import _lib
    import ctypes
    L = _lib.lib()
    g = torch.Generator(device='cuda').manual_seed(11)
    m = k = 200
    n = 700
    A = torch.randn(m, k, device='cuda', generator=g, dtype=F32)
    B = torch.randn(k, n, device='cuda', generator=g, dtype=F32)
    ref = A.double() @ B.double()
    Acm = A.T.contiguous()   # column-major A
    Bcm = B.T.contiguous()   # column-major B (k x n, ld k); the result lands here (ld m = k)
    wb = 256 + int(L.slab_sgemm_tc_work_bytes(m, n, k, 1))
    work = torch.empty(wb, dtype=torch.uint8, device='cuda')
    st = L.slab_sgemm_tc(m, n, k, 1.0, _lib.ptr(Acm), m, 0, _lib.ptr(Bcm), k, 0, 0.0, _lib.ptr(Bcm), m, 0, 1,
                         _lib.ptr(work), ctypes.c_size_t(wb), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(st, 'slab_sgemm_tc')
    out = Bcm.T.double()
    assert (torch.linalg.norm(out - ref) / torch.linalg.norm(ref)).item() < 1e-5


@pytest.mark.parametrize('precision', ['mixed', 'fp32'])
def test_engine_tree_schur_updates_on_tensor_cores(precision):
    """An engine whose merge tree forms its Schur updates on the tensor cores
    (SLAB_OPT_TREE_TC = 1) solves to the FP64 sparse-direct oracle like the
    CUDA-core tree (p = 22 leaves: merges with 80 and 160 eliminated unknowns)."""
    import numpy as np
    from oracle import domain as odomain
    from oracle import funcs as ofuncs
    from slablu_gb300 import _lib, hps
    from slablu_gb300.engine import SlabEngine
    geom, p, n, kh = [[0, 1], [0, 1]], 22, 160, 60.0   # 8 x 8 leaves
    a = 1 / (2 * (n / (p - 2)))
    md = odomain.Multidomain(geom, a, p)
    part = odomain.SlabPartition(md, 1.0)
    co = md.coeffs(ofuncs.helmholtz_pdo(lambda x: ofuncs.bfield_gaussian_bumps(x, kh)))
    ud = lambda x: ofuncs.uu_dir_greens(x, kh)
    ref = odomain.solve_full(md, part, co, ud)['sol_tot'][:, 0]
    g = hps.Geometry(geom, a, p, 1.0)
    coeffs = {k: torch.as_tensor(v.ravel(), device='cuda') for k, v in co.items() if v is not None}
    bnd = torch.as_tensor(ud(md.xx_active), device='cuda')
    for tc in (1, 0):
        eng = SlabEngine(g, precision)
        assert eng.L.slab_engine_set_option(eng.h, _lib.SLAB_OPT_TREE_TC, tc) == 0
        assert eng.L.slab_engine_get_option(eng.h, _lib.SLAB_OPT_TREE_TC) == tc
        eng.factor(**coeffs)
        u, _, iters, st = eng.solve(bnd, tol=1e-12, max_iter=40)
        assert st['converged']
        rel = float(np.linalg.norm(u[:, 0].cpu().numpy() - ref) / np.linalg.norm(ref))
        assert rel < 1e-9, (tc, rel, iters)
    e64 = SlabEngine(g, 'fp64')
    assert e64.L.slab_engine_set_option(e64.h, _lib.SLAB_OPT_TREE_TC, 1) != 0   # FP64 trees stay on FP64 cores
