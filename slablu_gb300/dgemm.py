"""FP64 GEMM on the tensor cores (slab_dgemm_emu) for device float64 tensors."""
import ctypes

import torch

from . import _lib


def dgemm_emu(A, B, C=None, alpha=1.0, beta=0.0):
    """alpha * A @ B + beta * C for CUDA float64 matrices, computed by exact
    BF16 slicing on the tensor cores (see include/slablu_gb300.h)."""
    L = _lib.lib()
    m, k = A.shape
    k2, n = B.shape
    if k != k2:
        raise ValueError('inner dimensions differ')
    At = A.T.contiguous()  # column-major storage of A
    Bt = B.T.contiguous()
    if C is None:
        Ct = torch.zeros(n, m, dtype=torch.float64, device=A.device)
        beta = 0.0
    else:
        Ct = C.T.contiguous()
    wb = int(L.slab_dgemm_emu_work_bytes(m, n, k))
    work = torch.empty(wb, dtype=torch.uint8, device=A.device)
    st = L.slab_dgemm_emu(m, n, k, float(alpha), _lib.ptr(At), m, _lib.ptr(Bt), k, float(beta), _lib.ptr(Ct), m,
                          _lib.ptr(work), ctypes.c_size_t(wb), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(st, 'slab_dgemm_emu')
    return Ct.T


def sgemm_tc(A, B, C=None, alpha=1.0, beta=0.0):
    """alpha * A @ B + beta * C for CUDA float32 matrices or batches (b, m, k) @ (b, k, n),
    on the TF32 tensor cores by exact three-way splitting (FP32 error bound; see
    include/slablu_gb300.h, slab_sgemm_tc)."""
    L = _lib.lib()
    batched = A.dim() == 3
    A3, B3 = (A, B) if batched else (A[None], B[None])
    bt, m, k = A3.shape
    bt2, k2, n = B3.shape
    if k != k2 or bt != bt2:
        raise ValueError('shapes do not match')
    f32 = torch.float32
    At = A3.transpose(1, 2).to(f32).contiguous()  # column-major storage of each A
    Bt = B3.transpose(1, 2).to(f32).contiguous()
    if C is None:
        Ct = torch.zeros(bt, n, m, dtype=f32, device=A.device)
        beta = 0.0
    else:
        Ct = (C if batched else C[None]).transpose(1, 2).to(f32).contiguous()
    wb = 256 + int(L.slab_sgemm_tc_work_bytes(m, n, k, bt))
    work = torch.empty(wb, dtype=torch.uint8, device=A.device)
    st = L.slab_sgemm_tc(m, n, k, float(alpha), _lib.ptr(At), m, m * k, _lib.ptr(Bt), k, k * n, float(beta),
                         _lib.ptr(Ct), m, m * n, bt, _lib.ptr(work), ctypes.c_size_t(wb),
                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(st, 'slab_sgemm_tc')
    out = Ct.transpose(1, 2)
    return out if batched else out[0]
