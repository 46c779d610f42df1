"""GPU test of slab_leaf_dtn_noalloc, the leaf DtN entry point that allocates nothing.

Callers that cannot allocate device memory at the point of use (an
application whose own pool allocator owns every device byte, or a program with
a device-memory budget fixed at start-up) get DtN maps from a scratch array
built into the library instead of a work buffer they pass in.  This file
checks, through the C ABI, that two calls in a row give the same maps as
slab_leaf_dtn with its own work buffer, that a call after the first one on the
device takes no device memory (free bytes and torch's allocation unchanged),
and that a batch too large for the built-in scratch is refused with a clear
error.  It is named to be collected last.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def lib():
    if not torch.cuda.is_available():
        pytest.fail('GPU test needs CUDA')
    from slablu_gb300 import build
    build.build()
    from slablu_gb300 import _lib
    return _lib


def _operands(p, nleaf, seed):
    from slablu_gb300 import hps
    ops = hps.LeafOps(0.01, p)
    rng = np.random.default_rng(seed)
    n = p * p
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device='cuda')
    co = [dev(1 + 0.2 * rng.random((nleaf, n))), dev(1 + 0.2 * rng.random((nleaf, n))), None, None,
          dev(-400.0 * (1 + rng.random((nleaf, n))))]
    return co, dev(ops.D), dev(ops.Dsq), dev(ops.Nx)


def _with_work(L, p, nleaf, co, D, Dsq, Nx, prec):
    q = p - 2
    wb = int(L.slab_leaf_dtn_work_bytes(nleaf, p, prec))
    work = torch.empty(wb, dtype=torch.uint8, device='cuda')
    dtn = torch.empty(nleaf, 4 * q, 4 * q, dtype=torch.float64, device='cuda')
    info = torch.zeros(nleaf, dtype=torch.int32, device='cuda')
    P = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
    st = L.slab_leaf_dtn(nleaf, p, *[P(c) for c in co], P(D), P(Dsq), P(Nx), prec, P(work), wb, P(dtn), None,
                         P(info), None)
    assert st == 0, L.slab_last_error()
    return dtn, info


def _no_alloc(L, p, nleaf, co, D, Dsq, Nx, prec):
    q = p - 2
    dtn = torch.empty(nleaf, 4 * q, 4 * q, dtype=torch.float64, device='cuda')
    info = torch.zeros(nleaf, dtype=torch.int32, device='cuda')
    P = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
    st = L.slab_leaf_dtn_noalloc(nleaf, p, *[P(c) for c in co], P(D), P(Dsq), P(Nx), prec, P(dtn), P(info), None)
    assert st == 0, L.slab_last_error()
    return dtn, info


@pytest.mark.parametrize('precision,tol', [(0, 1e-12), (2, 1e-6)])
def test_no_alloc_matches_work_buffer_entry_point(lib, precision, tol):
    L = lib.lib()
    p, nleaf = 12, 48
    assert L.slab_leaf_dtn_work_bytes(nleaf, p, precision) <= L.slab_leaf_dtn_noalloc_max_bytes()
    for call, seed in enumerate((11, 12)):  # two calls in a row share the scratch
        co, D, Dsq, Nx = _operands(p, nleaf, seed)
        ref, rinfo = _with_work(L, p, nleaf, co, D, Dsq, Nx, precision)
        got, ginfo = _no_alloc(L, p, nleaf, co, D, Dsq, Nx, precision)
        torch.cuda.synchronize()
        assert int(ginfo.abs().sum()) == 0 and int(rinfo.abs().sum()) == 0
        rel = (torch.linalg.norm(got - ref) / torch.linalg.norm(ref)).item()
        assert rel <= tol, (call, rel)


def test_no_alloc_call_takes_no_device_memory(lib):
    """After the first call on the device (which loads the library's kernels and
    looks up the scratch address), a call leaves the device's free memory and
    torch's allocations exactly as they were."""
    L = lib.lib()
    p, nleaf = 22, 16
    co, D, Dsq, Nx = _operands(p, nleaf, 21)
    _with_work(L, p, nleaf, co, D, Dsq, Nx, 2)
    _no_alloc(L, p, nleaf, co, D, Dsq, Nx, 2)     # first call on this device
    q = p - 2
    dtn = torch.empty(nleaf, 4 * q, 4 * q, dtype=torch.float64, device='cuda')
    info = torch.zeros(nleaf, dtype=torch.int32, device='cuda')
    P = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
    torch.cuda.synchronize()
    free0, alloc0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    st = L.slab_leaf_dtn_noalloc(nleaf, p, *[P(c) for c in co], P(D), P(Dsq), P(Nx), 2, P(dtn), P(info), None)
    torch.cuda.synchronize()
    assert st == 0, L.slab_last_error()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_allocated() == alloc0


def test_no_alloc_rejects_batches_beyond_its_scratch(lib):
    L = lib.lib()
    p = 22
    limit = L.slab_leaf_dtn_noalloc_max_bytes()
    nleaf = int(limit // L.slab_leaf_dtn_work_bytes(1, p, 0)) + 8
    co, D, Dsq, Nx = _operands(p, 1, 3)
    dtn = torch.empty(1, dtype=torch.float64, device='cuda')
    st = L.slab_leaf_dtn_noalloc(nleaf, p, *[None] * 5, ctypes.c_void_p(D.data_ptr()),
                                 ctypes.c_void_p(Dsq.data_ptr()), ctypes.c_void_p(Nx.data_ptr()), 0,
                                 ctypes.c_void_p(dtn.data_ptr()), None, None)
    assert st == -1
    assert b'scratch' in L.slab_last_error()
