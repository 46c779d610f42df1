"""The finite-difference discretisation: the oracle against the reference's own
grid, index sets, operator, slab partition and solution
(tests/golden/fd_n120_ppw20.npz, written by tests/golden/make_golden.py from
the reference's Domain_Solver with p = 0: 121 x 121 grid, constant Helmholtz at
20 points per wavelength, free-space Dirichlet data)."""
import hashlib
import os

import numpy as np
import pytest

from oracle import fd as ofd
from oracle import funcs


def test_fd_discretisation_and_solution_match_reference(golden_dir):
    g = np.load(os.path.join(golden_dir, 'fd_n120_ppw20.npz'))
    kh, h, stride = float(g['kh']), float(g['h']), int(g['stride'])
    pdo = funcs.helmholtz_pdo(lambda x: funcs.bfield_constant(x, kh))
    disc = ofd.FDDisc(g['box'], h, pdo)
    assert np.array_equal(disc.ns, g['ns'])
    assert np.array_equal(disc.XX[::stride], g['XX'])
    assert np.array_equal(disc.I_X, g['I_X'])
    A = disc.assemble_sparse().tocsr()
    A.sort_indices()
    assert A.nnz == int(g['A_nnz'])
    assert hashlib.sha256(A.indptr.astype(np.int64).tobytes()).hexdigest() == str(g['A_indptr_sha'])
    assert hashlib.sha256(A.indices.astype(np.int64).tobytes()).hexdigest() == str(g['A_indices_sha'])
    assert np.array_equal(A.data[::stride], g['A_data_sub'])
    part = ofd.FDPartition(disc, float(g['buf_constant']))
    assert (part.buf, part.buf_prime, part.Npan, part.Npan_loc) == tuple(
        int(g[k]) for k in ('buf', 'buf_prime', 'Npan', 'Npan_loc'))
    assert np.array_equal(part.inds_pans, g['inds_pans'])
    for nm in ('I_L', 'I_R', 'I_D', 'I_U', 'I_C', 'I_Ctot', 'I_Xtot'):
        assert np.array_equal(getattr(part, nm), g[nm]), nm
    ud = lambda x: funcs.uu_dir_greens(x, kh)
    sol, res = ofd.solve(disc, part, A, ud)
    ref = g['superLU_sol_sub']
    assert np.linalg.norm(sol[::stride] - ref) / np.linalg.norm(ref) < 1e-12
    assert res < 1e-13
    true = ud(disc.XX)
    trueres = np.linalg.norm(sol - true) / np.linalg.norm(true)
    assert abs(trueres - float(g['superLU_trueres'])) < 1e-9 * float(g['superLU_trueres'])
    # the reference's slab solver gives the same solution
    refs = g['slabLU_sol_sub']
    assert np.linalg.norm(sol[::stride] - refs) / np.linalg.norm(refs) < 1e-11


def test_fd_rejects_the_reference_broken_c2_term():
    pdo = dict(funcs.helmholtz_pdo(lambda x: funcs.bfield_constant(x, 5.0)))
    pdo['c2'] = lambda x: np.ones(x.shape[0])
    with pytest.raises(ValueError):
        ofd.FDDisc([[0, 1], [0, 1]], 0.1, pdo).assemble_sparse()
