"""CPU tests of the product's host logic and of the C-ABI library boundary."""
import ctypes
import os

import numpy as np
import pytest

from oracle import domain as odomain
from oracle import leaf as oleaf
from slablu_gb300 import _lib, hps


@pytest.mark.parametrize('p,a', [(6, 0.1), (8, 0.0125), (12, 0.0125), (16, 1 / 144), (22, 0.005)])
def test_leaf_ops_match_oracle(p, a):
    ops = hps.LeafOps(a, p)
    ld = oleaf.leaf_disc(a, p)
    for nm in ('Jl', 'Jr', 'Jd', 'Ju', 'Jx', 'Jc', 'Jxreorder'):
        assert np.array_equal(getattr(ops, nm), getattr(ld, nm)), nm
    assert np.array_equal(ops.zz, ld.zz)
    assert np.array_equal(ops.D, ld.D)
    assert np.abs(ops.Nx - ld.Nx).max() == 0.0
    assert np.abs(ops.Interp_mat - ld.Interp_mat).max() <= 1e-12
    # Kronecker operators the kernels build on the fly from D and Dsq
    assert np.array_equal(np.kron(ops.Dsq, np.eye(p)), ld.D11)
    assert np.array_equal(np.kron(np.eye(p), ops.Dsq), ld.D22)


@pytest.mark.parametrize('geom,p,n', [([[0, 1], [0, 1]], 8, 48), ([[0, 1], [0, 1]], 12, 400),
                                      ([[0, 1], [0, 0.5]], 8, 48), ([[0, 1], [0, 1]], 22, 400)])
def test_geometry_and_partition_match_oracle(geom, p, n):
    a = 1 / (2 * (n / (p - 2)))
    g = hps.Geometry(geom, a, p, 1.0)
    md = odomain.Multidomain(geom, a, p)
    part = odomain.SlabPartition(md, 1.0)
    assert (g.n0, g.n1) == (md.n0, md.n1) and g.ntot == md.ntot
    assert np.array_equal(g.xx, md.xx)
    assert np.array_equal(g.leafglob, md.face_index())
    assert np.array_equal(g.xx_active, md.xx_active)
    assert g.buf == part.buf and g.Npan == part.Npan
    for nm in ('I_L', 'I_R', 'I_D', 'I_U', 'I_C', 'I_Ctot', 'I_Xtot', 'inds_pans'):
        assert np.array_equal(getattr(g, nm), getattr(part, nm)), nm


def test_nearest_divisor():
    for nval in (1, 7, 12, 71, 100, 360):
        for x in range(1, 30):
            assert hps.nearest_divisor(nval, x) == odomain.nearest_divisor(nval, x)


def test_reported_unknowns():
    g = hps.Geometry([[0, 1], [0, 1]], 1 / (2 * 100), 22)
    assert g.N_reported == 4404000


def test_library_exports_every_declared_symbol():
    if not os.path.exists(_lib.LIB_PATH):
        from slablu_gb300 import build
        build.build()
    L = ctypes.CDLL(_lib.LIB_PATH)
    syms = _lib.header_symbols()
    assert len(syms) >= 10
    for s in syms:
        assert hasattr(L, s), s
    lib = _lib.lib()
    assert lib.slab_version() >= 100
    # argument validation runs without a GPU
    h = ctypes.c_void_p()
    z = np.zeros(4)
    st = lib.slab_engine_create(ctypes.byref(h), 1, 1, 1, 1, 1, _lib.np_ptr(z, ctypes.c_double),
                                _lib.np_ptr(z, ctypes.c_double), _lib.np_ptr(z, ctypes.c_double),
                                _lib.np_ptr(z, ctypes.c_double), _lib.np_ptr(np.zeros(4, np.int32), ctypes.c_int),
                                None)
    assert st == -1
    assert b'invalid' in lib.slab_last_error()
    assert lib.slab_leaf_dtn_work_bytes(0, 22, 0) == 0
    assert lib.slab_leaf_dtn_work_bytes(10, 22, 0) > 10 * 400 * 480 * 8
    # the mixed-derivative entry points: 4(p-1) extra columns and the interpolation matrix
    assert lib.slab_leaf_dtn_mixed_work_bytes(0, 22, 0) == 0
    assert lib.slab_leaf_dtn_mixed_work_bytes(10, 22, 0) >= lib.slab_leaf_dtn_work_bytes(10, 22, 0) + \
        10 * 400 * 4 * 8 + 84 * 80 * 8
    st = lib.slab_engine_create_mixed(ctypes.byref(h), 1, 1, 1, 1, 1, _lib.np_ptr(z, ctypes.c_double),
                                      _lib.np_ptr(z, ctypes.c_double), _lib.np_ptr(z, ctypes.c_double),
                                      _lib.np_ptr(z, ctypes.c_double), _lib.np_ptr(np.zeros(4, np.int32), ctypes.c_int),
                                      None)
    assert st == -1
    assert lib.slab_engine_factor_mixed(None, None, None, None, None, None, None) == -1
    assert b'null engine' in lib.slab_last_error()
    assert lib.slab_leaf_dtn_mixed(4, 22, *([None] * 11), 0, None, 0, None, None, None, None) == -1
    assert lib.slab_csr_assemble(-1, None, None, 0, None, None) == -1
    assert lib.slab_csr_spmv(-1, None, None, None, None, 1.0, 0.0, None, None) == -1


@pytest.mark.parametrize('geom,p,n', [([[0, 1], [0, 1]], 8, 48), ([[0, 1], [0, 0.5]], 6, 28)])
def test_reduced_pattern_matches_oracle_csr(geom, p, n):
    """The device assembly's CSR pattern and slot map reproduce SciPy's COO -> CSR sum of
    the leaf DtN maps (hps_multidomain_disc.py:84-95), here with random DtN values."""
    from slablu_gb300 import sparse
    a = 1 / (2 * (n / (p - 2)))
    md = odomain.Multidomain(geom, a, p)
    g = hps.Geometry(geom, a, p, 1.0)
    indptr, indices, dest = sparse.reduced_pattern(g)
    rng = np.random.default_rng(3)
    dtn = rng.standard_normal((md.nboxes, 4 * md.q, 4 * md.q))
    ref = md.sparse_mat(dtn)
    ref.sort_indices()
    assert np.array_equal(indptr, ref.indptr) and np.array_equal(indices, ref.indices)
    vals = np.zeros(len(indices))
    np.add.at(vals, dest, dtn.ravel())
    assert np.array_equal(vals, ref.data)
