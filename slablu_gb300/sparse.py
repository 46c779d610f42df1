"""Reduced sparse operator of the HPS discretisation on the device.

Mirrors HPS_Multidomain.sparse_mat (src_disc/hps_multidomain_disc.py:53-109):
the leaf DtN maps summed over the reduced face unknowns, as a CSR matrix, and
the sparse applies of the right-hand-side formation
(src_solver/slablu_solver.py:48-57, :489-507).  The reference builds the COO
triplets with Python loops and lets SciPy sort and sum them on the host; here
the pattern (fixed by the leaf grid) is built once with NumPy and cached on the
geometry, and the values are summed on the GPU by slab_csr_assemble
(include/slablu_gb300.h).  The factor-and-solve path does not need this
operator; it exists for callers of the reference's sparse interface.
"""
import ctypes

import numpy as np
import torch

from . import _lib


def reduced_pattern(geom):
    """CSR pattern of the reduced operator and the slot of every leaf DtN entry.

    Returns (indptr int64 (ntot+1,), indices int32 (nnz,), dest int64
    (nleaf * nx * nx,)), NumPy arrays, cached on ``geom``.  Entry (r, c) of leaf
    l's DtN (row-major) lands in slot dest[(l * nx + r) * nx + c]; columns are
    sorted within each row, as SciPy's canonical CSR.
    """
    cached = getattr(geom, '_reduced_pattern', None)
    if cached is not None:
        return cached
    idx = np.asarray(geom.leafglob, dtype=np.int64)
    ntot = int(geom.ntot)
    keys = (idx[:, :, None] * ntot + idx[:, None, :]).ravel()
    uniq, dest = np.unique(keys, return_inverse=True)
    rows, cols = uniq // ntot, uniq % ntot
    indptr = np.zeros(ntot + 1, dtype=np.int64)
    indptr[1:] = np.cumsum(np.bincount(rows, minlength=ntot))
    out = (indptr, cols.astype(np.int32), dest.reshape(-1).astype(np.int64))
    geom._reduced_pattern = out
    return out


class ReducedCSR:
    """Device CSR matrix (FP64) with the product y = alpha A x + beta y."""

    def __init__(self, indptr, indices, vals, shape):
        self.indptr, self.indices, self.vals, self.shape = indptr, indices, vals, shape

    @property
    def nnz(self):
        return int(self.vals.numel())

    def to_torch(self):
        return torch.sparse_csr_tensor(self.indptr, self.indices, self.vals, size=self.shape)

    def matvec(self, x, alpha=1.0, beta=0.0, y=None):
        """alpha A x (+ beta y); x (ncols,) or (ncols, k) FP64 on the matrix's device."""
        L = _lib.lib()
        x = x.to(torch.float64)
        squeeze = x.dim() == 1
        X = x[:, None] if squeeze else x
        if y is None:
            Y = torch.zeros(self.shape[0], X.shape[1], dtype=torch.float64, device=X.device)
            beta = 0.0
        else:
            Y = y[:, None] if y.dim() == 1 else y
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        for j in range(X.shape[1]):
            xj = X[:, j].contiguous()
            yj = Y[:, j].contiguous()
            _lib.check(L.slab_csr_spmv(self.shape[0], _lib.ptr(self.indptr), _lib.ptr(self.indices),
                                       _lib.ptr(self.vals), _lib.ptr(xj), float(alpha), float(beta), _lib.ptr(yj),
                                       stream), 'slab_csr_spmv')
            Y[:, j] = yj
        return Y[:, 0] if squeeze else Y


def row_subset(geom, A, rows):
    """The rows ``rows`` (reduced indices) of the reduced operator ``A`` as a CSR
    matrix (len(rows) x ntot) sharing A's values (gathered on the device)."""
    indptr, indices, _ = reduced_pattern(geom)
    rows = np.asarray(rows, dtype=np.int64)
    lens = indptr[rows + 1] - indptr[rows]
    sub_ptr = np.zeros(rows.size + 1, dtype=np.int64)
    sub_ptr[1:] = np.cumsum(lens)
    slots = np.repeat(indptr[rows] - sub_ptr[:-1], lens) + np.arange(int(sub_ptr[-1]))
    dev = A.vals.device
    sl = torch.as_tensor(slots, device=dev)
    return ReducedCSR(torch.as_tensor(sub_ptr, device=dev), torch.as_tensor(indices[slots], device=dev),
                      A.vals[sl].contiguous(), (int(rows.size), A.shape[1]))


def assemble(geom, dtn):
    """Reduced operator from leaf DtN maps ``dtn`` (nleaf, nx, nx) FP64 on the GPU."""
    L = _lib.lib()
    indptr, indices, dest = reduced_pattern(geom)
    dev = dtn.device
    nleaf, nx = int(geom.nboxes), 4 * int(geom.q)
    if tuple(dtn.shape) != (nleaf, nx, nx):
        raise ValueError(f'dtn has shape {tuple(dtn.shape)}, expected {(nleaf, nx, nx)}')
    src = dtn.to(torch.float64).contiguous()
    dest_d = torch.as_tensor(dest, device=dev)
    vals = torch.empty(len(indices), dtype=torch.float64, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(L.slab_csr_assemble(src.numel(), _lib.ptr(src), _lib.ptr(dest_d), vals.numel(), _lib.ptr(vals),
                                   stream), 'slab_csr_assemble')
    return ReducedCSR(torch.as_tensor(indptr, device=dev), torch.as_tensor(indices, device=dev), vals,
                      (int(geom.ntot), int(geom.ntot)))
