"""FP64 GEMM emulated on the BF16 tensor cores against cuBLAS FP64 (through torch).

Error bound per entry: about k 2^-53 max|A(i,:)| max|B(:,j)|; the tests check
the normwise relative error against that scale with a 4x margin.
"""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.fail('GPU tests need CUDA')
    from slablu_gb300 import build
    build.build()


def _check(A, B, C=None, alpha=1.0, beta=0.0):
    from slablu_gb300.dgemm import dgemm_emu
    ref = alpha * (A @ B) + (beta * C if C is not None else 0.0)
    out = dgemm_emu(A, B, None if C is None else C.clone(), alpha=alpha, beta=beta)
    k = A.shape[1]
    scale = A.abs().amax(dim=1, keepdim=True) * B.abs().amax(dim=0, keepdim=True)
    err = ((out - ref).abs() / (scale * abs(alpha) + 1e-300)).max().item()
    assert err <= 4 * k * 2.0 ** -53, err
    return out, ref


@pytest.mark.parametrize('m,n,k', [(128, 32, 256), (200, 70, 300), (512, 512, 1000), (1000, 333, 2001)])
def test_dgemm_emu_random(m, n, k):
    g = torch.Generator(device='cuda').manual_seed(m + n + k)
    A = torch.randn(m, k, dtype=torch.float64, device='cuda', generator=g)
    B = torch.randn(k, n, dtype=torch.float64, device='cuda', generator=g)
    out, ref = _check(A, B)
    rel = (torch.linalg.norm(out - ref) / torch.linalg.norm(ref)).item()
    assert rel < 4e-15, rel  # both products carry rounding error; FP64 unit roundoff is 1.1e-16


def test_dgemm_emu_scaled_rows_and_beta():
    g = torch.Generator(device='cuda').manual_seed(7)
    m, n, k = 300, 96, 700
    A = torch.randn(m, k, dtype=torch.float64, device='cuda', generator=g)
    A *= torch.logspace(-30, 30, m, dtype=torch.float64, device='cuda')[:, None]
    A[5] = 0.0
    B = torch.randn(k, n, dtype=torch.float64, device='cuda', generator=g)
    B *= torch.logspace(20, -20, n, dtype=torch.float64, device='cuda')[None, :]
    C = torch.randn(m, n, dtype=torch.float64, device='cuda', generator=g)
    out, ref = _check(A, B, C, alpha=-1.0, beta=1.0)
    assert torch.equal(out[5], C[5])


def test_dgemm_emu_nonfinite_rows_give_nan():
    from slablu_gb300.dgemm import dgemm_emu
    A = torch.ones(130, 64, dtype=torch.float64, device='cuda')
    A[3, 7] = float('inf')
    B = torch.ones(64, 40, dtype=torch.float64, device='cuda')
    out = dgemm_emu(A, B)
    assert torch.isnan(out[3]).all()
    assert torch.equal(out[4], torch.full((40,), 64.0, dtype=torch.float64, device='cuda'))
