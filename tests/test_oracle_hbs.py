"""HBS compression from sketches: the oracle against the reference's own results.

tests/golden/hbs.npz was written by tests/golden/make_golden.py with the
reference's HBS_matrix (src_solver/hbs_reconstruction.py) on small test
operators: three levels (m = 8 leaf blocks), one level (m = 2), and a leaf
count padded from 6 to 8 (the padding sketches the reference draws are
replayed).  The bases of a level are fixed by the sketches only up to
directions with noise-level singular values, so the pins are the represented
matrix -- products with it and its transpose, the compressed inverse, the dense
form -- and, where the bases are well determined (one level), the stored
diagonal blocks.
"""
import os

import numpy as np
import pytest

from oracle import hbs

TAGS = ['L3', 'L1', 'pad']


def _rel(a, r):
    return np.linalg.norm(a - r) / np.linalg.norm(r)


def _operator(x, b):
    d = np.abs(x[:, None] - x[None, :])
    return np.stack([(1.0 + 0.3 * j) / (1.0 + 40.0 * d) + (2.0 + j) * np.eye(x.size) for j in range(b)])


@pytest.mark.parametrize('tag', TAGS)
def test_hbs_reconstruction_matches_reference(golden_dir, tag):
    g = np.load(os.path.join(golden_dir, 'hbs.npz'))
    b, n, k, bs, m, n_pad, L = [int(v) for v in g[tag + '_shape']]
    H = hbs.HBSMatrix(b, n, k)
    assert (H.bs, H.m, H.n_pad) == (bs, m, n_pad)
    kw = dict(Omega_pad=g[tag + '_Om_pad'], Psi_pad=g[tag + '_Ps_pad']) if n_pad else {}
    H.reconstruct(g[tag + '_Om'], g[tag + '_Ps'], g[tag + '_Y'], g[tag + '_Z'], **kw)
    assert H.L == L
    assert _rel(H.matvec(g[tag + '_q']), g[tag + '_mv']) < 1e-11
    assert _rel(H.matvec(g[tag + '_q'], transpose=True), g[tag + '_mvT']) < 1e-11
    dense = H.todense()
    assert np.abs(np.einsum('bij,bjr->bir', dense, g[tag + '_q']) - H.matvec(g[tag + '_q'])).max() < 1e-12 * \
        np.abs(g[tag + '_mv']).max()
    if tag + '_D' in g.files:
        assert _rel(H.D, g[tag + '_D']) < 1e-12
        assert _rel(dense, g[tag + '_dense']) < 1e-12
    # the compression approximates the sketched operator
    A = _operator(g[tag + '_x'], b)
    assert _rel(dense, A) < 0.05
    H.calc_inverse()
    assert _rel(H.apply_inverse(g[tag + '_f']), g[tag + '_inv']) < 1e-11
    assert _rel(H.apply_inverse(g[tag + '_f'], transpose=True), g[tag + '_invT']) < 1e-11
    # the compressed inverse inverts the compressed matrix
    X = H.apply_inverse(g[tag + '_f'])
    assert _rel(np.einsum('bij,bjr->bir', dense, X), g[tag + '_f']) < 1e-10


def test_block_size_rule():
    assert hbs.nearest_div_up(200, 120) == 200
    assert hbs.nearest_div_up(400, 136) == 200
    H = hbs.HBSMatrix(1, 96, 8)
    assert (H.bs, H.m, H.n_pad) == (16, 8, 32)
