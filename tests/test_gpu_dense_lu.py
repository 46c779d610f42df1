"""Dense FP64 LU of the C ABI (slab_dense_lu / slab_dense_lu_solve), the
factorization of the periodic edge's Schur complement, against an FP64
reference solve (torch on the GPU) and the residual."""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.fail('GPU tests need CUDA')
    from slablu_gb300 import build
    build.build()


@pytest.mark.parametrize('n,nrhs', [(1, 1), (31, 2), (300, 5), (1000, 3), (2000, 8)])
def test_dense_lu_solves(n, nrhs):
    from slablu_gb300.periodic import DenseLU
    g = torch.Generator(device='cuda').manual_seed(n)
    A = torch.randn(n, n, dtype=torch.float64, device='cuda', generator=g)
    A += torch.diag(torch.linspace(-3.0, 3.0, n, dtype=torch.float64, device='cuda'))   # indefinite, pivoting matters
    B = torch.randn(n, nrhs, dtype=torch.float64, device='cuda', generator=g)
    X = DenseLU(A).solve(B)
    ref = torch.linalg.solve(A, B)
    assert (torch.linalg.norm(X - ref) / torch.linalg.norm(ref)).item() < 1e-10
    res = torch.linalg.norm(A @ X - B) / (torch.linalg.norm(A) * torch.linalg.norm(X))
    assert res.item() < 1e-14
    x1 = DenseLU(A).solve(B[:, 0])
    assert x1.shape == (n,) and torch.allclose(x1, X[:, 0], rtol=0, atol=1e-12 * float(X.abs().max()))


def test_dense_lu_reports_a_zero_pivot():
    from slablu_gb300 import _lib
    from slablu_gb300.periodic import DenseLU
    A = torch.zeros(40, 40, dtype=torch.float64, device='cuda')
    A[:20, :20] = torch.eye(20, dtype=torch.float64, device='cuda')
    with pytest.raises(_lib.SlabError) as e:
        DenseLU(A)
    assert e.value.status == 21
