"""Generate golden vectors by running the reference (annayesy/slabLU) itself.

Run in a container where the reference source is mounted, giving its path:

    python tests/golden/make_golden.py REFERENCE_DIR [mode]

The reference needs SciPy sparse indexing to accept torch index tensors
(SciPy >= 1.11 rejects them).  This script installs that conversion as a
monkeypatch in its own process; the reference source is not modified.
Outputs are small .npz files beside this script; they are committed and read
by the CPU tests (the reference source is not needed afterwards).
"""
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if len(sys.argv) < 2:
    sys.exit('usage: make_golden.py REFERENCE_DIR [mode]')
REF = sys.argv[1]
os.environ['CUDA_VISIBLE_DEVICES'] = ''

import torch  # noqa: E402
import scipy.sparse._index as _sp_index  # noqa: E402

torch.set_default_dtype(torch.double)
_get, _set = _sp_index.IndexMixin.__getitem__, _sp_index.IndexMixin.__setitem__


def _np_key(k):
    if isinstance(k, torch.Tensor):
        return k.numpy()
    if isinstance(k, tuple):
        return tuple(_np_key(x) for x in k)
    return k


_sp_index.IndexMixin.__getitem__ = lambda self, k: _get(self, _np_key(k))
_sp_index.IndexMixin.__setitem__ = lambda self, k, v: _set(self, _np_key(k), v)
sys.path.insert(0, REF)

from src_disc.hps_subdomain_disc import HPS_Disc  # noqa: E402
from src_disc import hps_parallel_leaf_ops as leaf_ops  # noqa: E402
from src_disc import hps_multidomain_disc  # noqa: E402
from src_disc import pdo as ref_pdo  # noqa: E402
import src_disc.built_in_funcs as bif  # noqa: E402
import src_solver.block_tridiag_solver_dense as ref_bt  # noqa: E402
from src_solver.slablu_solver import Domain_Solver  # noqa: E402


def save(name, **arrs):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrs)
    print('wrote', name, sum(v.nbytes for v in map(np.asarray, arrs.values())) // 1024, 'KiB')


def bumps32(xx, seed=0):
    """b = 1 + 0.5 sum of 32 Gaussian bumps (width 0.02) at seeded centres."""
    rng = np.random.default_rng(seed)
    cen = rng.random((32, 2))
    x = np.asarray(xx)
    d2 = ((x[:, None, :] - cen[None]) ** 2).sum(-1)
    return 1.0 + 0.5 * np.exp(-d2 / (2 * 0.02 ** 2)).sum(1)


def leaf_fixtures():
    for p, a in ((8, 0.0125), (12, 0.0125), (22, 0.005), (16, 1 / (2 * 71))):
        H = HPS_Disc(a, p, 2)
        J = H.JJ
        extra = {}
        if p <= 12:
            extra = dict(D1=H.Ds.D1, D2=H.Ds.D2, D11=H.Ds.D11, D22=H.Ds.D22)
        save(f'leaf_p{p}.npz', p=p, a=a, zz=H.zz, Jl=J.Jl, Jr=J.Jr, Jd=J.Jd, Ju=J.Ju,
             Jx=J.Jx, Jc=J.Jc, Jxreorder=J.Jxreorder, Nx=H.Nx, Interp_mat=H.Interp_mat, **extra)


def dtn_fixture(p, a, nbox_side, picks, kh, name, seed=0):
    """Reference form_DtNs (build and solve) on selected leaves of a grid."""
    md = hps_multidomain_disc.HPS_Multidomain(
        ref_pdo.PDO_2d(ref_pdo.ones, ref_pdo.ones), torch.tensor([[0, 1.0], [0, 1.0]]), a, p)
    xx = md.grid_xx[picks].clone()
    cvals = torch.tensor(-(kh ** 2) * bumps32(xx.reshape(-1, 2).numpy(), seed)).reshape(len(picks), -1)
    lut = {}

    def cfun(x):
        key = x.shape[0]
        return lut[key]

    lut[len(picks) * p * p] = cvals.reshape(-1)
    op = ref_pdo.PDO_2d(ref_pdo.ones, ref_pdo.ones, c=cfun)
    H = md.H
    Nx = torch.tensor(H.Nx)
    Jx = torch.tensor(H.JJ.Jx)
    Jc = torch.tensor(H.JJ.Jc)
    Jxr = torch.tensor(H.JJ.Jxreorder)
    Im = torch.tensor(H.Interp_mat)
    dev = torch.device('cpu')
    DtN = leaf_ops.form_DtNs(p, 2, xx, Nx, Jx, Jc, Jxr, H.Ds, Im, op, 0, len(picks), dev,
                             'build', torch.zeros(len(picks), 4 * (p - 2), 1), None)
    rng = np.random.default_rng(seed + 1)
    uface = torch.tensor(rng.standard_normal((len(picks), 4 * (p - 2), 2)))
    usol = leaf_ops.form_DtNs(p, 2, xx, Nx, Jx, Jc, Jxr, H.Ds, Im, op, 0, len(picks), dev,
                              'solve', uface, None)
    save(name, p=p, a=a, kh=kh, picks=np.asarray(picks), xx=xx.numpy(), c=cvals.numpy(),
         dtn=DtN.numpy(), u_face=uface.numpy(), u_solve=usol.numpy())


def smooth_coeffs(x, kh):
    """Variable coefficients with a mixed-derivative term, of the kind a curved
    domain's parameter map produces (src_disc/pdo.py:133-310)."""
    x0, x1 = x[:, 0], x[:, 1]
    return dict(c11=1.0 + 0.3 * np.sin(3 * x0) * np.cos(2 * x1), c22=1.0 + 0.2 * np.cos(2 * x0 + x1),
                c12=0.15 * np.sin(2 * x0) * np.cos(3 * x1), c1=0.5 * np.cos(x0 + 2 * x1),
                c2=-0.4 * np.sin(x0 * x1), c=-(kh ** 2) * (1.0 - 0.3 * np.exp(-((x0 - 0.5) ** 2 + (x1 - 0.5) ** 2) / 0.05)))


def dtn_c12_fixture(p, a, nbox_side, picks, kh, name, seed=0):
    """Reference form_DtNs (build and solve) with every coefficient present,
    including c12 (the Jxreorder / Interp_mat branch, hps_parallel_leaf_ops.py:59-65, 84-88)."""
    md = hps_multidomain_disc.HPS_Multidomain(
        ref_pdo.PDO_2d(ref_pdo.ones, ref_pdo.ones), torch.tensor([[0, 1.0], [0, 1.0]]), a, p)
    xx = md.grid_xx[picks].clone()
    vals = smooth_coeffs(xx.reshape(-1, 2).numpy(), kh)
    npts = len(picks) * p * p
    fn = {k: (lambda key: (lambda x: torch.tensor(vals[key]) if x.shape[0] == npts else None))(k) for k in vals}
    op = ref_pdo.PDO_2d(fn['c11'], fn['c22'], c12=fn['c12'], c1=fn['c1'], c2=fn['c2'], c=fn['c'])
    H = md.H
    Nx = torch.tensor(H.Nx)
    Jx = torch.tensor(H.JJ.Jx)
    Jc = torch.tensor(H.JJ.Jc)
    Jxr = torch.tensor(H.JJ.Jxreorder)
    Im = torch.tensor(H.Interp_mat)
    dev = torch.device('cpu')
    DtN = leaf_ops.form_DtNs(p, 2, xx, Nx, Jx, Jc, Jxr, H.Ds, Im, op, 0, len(picks), dev,
                             'build', torch.zeros(len(picks), 4 * (p - 2), 1), None)
    rng = np.random.default_rng(seed + 1)
    uface = torch.tensor(rng.standard_normal((len(picks), 4 * (p - 2), 2)))
    usol = leaf_ops.form_DtNs(p, 2, xx, Nx, Jx, Jc, Jxr, H.Ds, Im, op, 0, len(picks), dev,
                              'solve', uface, None)
    save(name, p=p, a=a, kh=kh, picks=np.asarray(picks), xx=xx.numpy(),
         **{k: v.reshape(len(picks), -1) for k, v in vals.items()},
         dtn=DtN.numpy(), u_face=uface.numpy(), u_solve=usol.numpy())


def assembly_fixture():
    p, a = 8, 0.0125
    geom = torch.tensor([[0, 4 * 2 * a], [0, 3 * 2 * a]])
    kh = 25.0
    op = ref_pdo.PDO_2d(ref_pdo.ones, ref_pdo.ones, c=lambda xx: bif.bfield_gaussian_bumps(xx, kh).reshape(-1))
    md = hps_multidomain_disc.HPS_Multidomain(op, geom, a, p)
    A, _ = md.sparse_mat(torch.device('cpu'))
    A.sort_indices()
    save('assembly_p8.npz', p=p, a=a, kh=kh, box_geom=geom.numpy(), data=A.data, indices=A.indices,
         indptr=A.indptr, shape=np.array(A.shape), I_unique=md.I_unique.numpy(),
         I_copy1=md.I_copy1.numpy(), I_copy2=md.I_copy2.numpy(), xx_active=md.xx_active.numpy(),
         xx_tot=md.xx_tot.numpy())


def partition_fixture():
    out = {}
    for (p, n) in ((8, 48), (12, 400), (22, 400), (22, 2000), (22, 1000), (16, 994)):
        a = 1 / (2 * (n / (p - 2)))
        op = ref_pdo.PDO_2d(ref_pdo.ones, ref_pdo.ones)
        dom = Domain_Solver(torch.tensor([[0, 1.0], [0, 1.0]]), op, 0.0, a, p=p, buf_constant=1.0)
        tag = f'p{p}_n{n}'
        out[tag + '_buf'] = np.array(dom.buf_pans)
        out[tag + '_Npan'] = np.array(dom.Npan)
        out[tag + '_nbox'] = dom.hps.n.numpy()
        for nm in ('I_C', 'I_L', 'I_R', 'I_D', 'I_U', 'I_Ctot', 'I_Xtot'):
            out[tag + '_' + nm] = np.asarray(getattr(dom, nm))
    save('partition.npz', **out)


def blocktri_fixture():
    rng = np.random.default_rng(7)
    out = {}
    for (b, m, bs) in ((3, 5, 4), (2, 7, 6), (4, 2, 3)):
        diag = torch.tensor(rng.standard_normal((b, m, bs, bs)) + 3 * np.eye(bs))
        sub = torch.tensor(rng.standard_normal((b, m - 1, bs, bs)))
        sup = torch.tensor(rng.standard_normal((b, m - 1, bs, bs)))
        f = torch.tensor(rng.standard_normal((b, m * bs, 3)))
        T = ref_bt.Block_Tridiagonal(b, m, bs)
        T.build_sweep(diag.clone(), sub.clone(), sup.clone(), fast_LU=False)
        x = T.lusolve_sweep(f.clone())
        xt = T.lusolve_sweep(f.clone(), transpose=True)
        tag = f'b{b}_m{m}_bs{bs}'
        so, po = m, m + (m - 1)
        out[tag + '_diag'] = diag.numpy(); out[tag + '_sub'] = sub.numpy(); out[tag + '_sup'] = sup.numpy()
        out[tag + '_f'] = f.numpy(); out[tag + '_x'] = x.numpy(); out[tag + '_xt'] = xt.numpy()
        out[tag + '_LU'] = T.Tdata[:, :so].numpy(); out[tag + '_Lsub'] = T.Tdata[:, so:po].numpy()
        out[tag + '_Usup'] = T.Tdata[:, po:po + m - 1].numpy()
        out[tag + '_piv'] = ref_bt.unpack_pivs(b, m, bs, T.Tdata, torch.device('cpu')).numpy()
    save('blocktri.npz', **out)


def run_domain(p, n, ppw, pde, solver, bc='free_space'):
    nwaves = int(n / ppw)
    kh = (nwaves + 0.03) * 2 * np.pi + 1.8
    if pde == 'bfield_constant':
        cf = lambda xx: bif.bfield_constant(xx, kh)
    else:
        cf = lambda xx: bif.bfield_gaussian_bumps(xx, kh).reshape(-1)
    op = ref_pdo.PDO_2d(ref_pdo.ones, ref_pdo.ones, c=cf)
    a = 1 / (2 * (n / (p - 2)))
    dom = Domain_Solver(torch.tensor([[0, 1.0], [0, 1.0]]), op, kh, a, p=p, buf_constant=1.0)
    dom.build('reduced_cpu', solver, verbose=False)
    if bc == 'free_space':
        uu = lambda xx: bif.uu_dir_func_greens(xx, kh)
    else:
        uu = lambda xx: torch.ones(xx.shape[0], 1)
    sol, res, tres, rloc, _ = dom.solve(uu, None, known_sol=(bc == 'free_space'))
    sol, res, tres, rloc, _ = dom.solve(uu, None, known_sol=(bc == 'free_space'))
    return dom, kh, sol.numpy(), float(res), float(tres), float(rloc)


def annulus_fixture(p=22, n=400, ppw=40):
    """The reference's annulus known-answer test (tests/test_2d.py:51-52): the
    parameter map of the annulus (src_disc/pdo.py:196-215) turns Helmholtz on the
    annulus into a variable-coefficient operator with a mixed derivative on the
    unit square; Dirichlet data is the free-space Green's function at the mapped
    points (argparse_driver.py:195-203)."""
    nwaves = int(n / ppw)
    kh = (nwaves + 0.03) * 2 * np.pi + 1.8
    op, param_map, _ = ref_pdo.get_param_map_and_pdo('annulus', bif.bfield_constant, kh)
    a = 1 / (2 * (n / (p - 2)))
    dom = Domain_Solver(torch.tensor([[0, 1.0], [0, 1.0]]), op, kh, a, p=p, buf_constant=1.0)
    dom.build('reduced_cpu', 'slabLU', verbose=False)
    uu = lambda xx: bif.uu_dir_func_greens(param_map(xx), kh)
    sol, res, tres, rloc, _ = dom.solve(uu, None, known_sol=True)
    sol, res, tres, rloc, _ = dom.solve(uu, None, known_sol=True)
    xx = dom.hps.xx_tot
    pick = np.arange(0, xx.shape[0], 97)
    xs = xx[pick]
    coef = {k: (np.zeros(xs.shape[0]) if getattr(op, k) is None else np.asarray(getattr(op, k)(xs)).reshape(-1))
            for k in ('c11', 'c22', 'c12', 'c1', 'c2', 'c')}
    stride = 7
    save(f'annulus_p{p}_n{n}_ppw{ppw}.npz', p=p, n=n, ppw=ppw, kh=kh, stride=stride,
         sol_sub=sol.numpy()[::stride], sol_norm=np.linalg.norm(sol.numpy()), res=float(res),
         trueres=float(tres), resloc=float(rloc), coef_pick=pick, coef_xx=xs.numpy(),
         mapped_xx=param_map(xs).numpy(), **{'coef_' + k: v for k, v in coef.items()})


def periodic_fixture(name, geom, box, p, n, ppw, stride=5):
    """Periodic boundary (Domain_Solver(periodic_bc=True)): the left and right
    edges of the rectangle are identified, Dirichlet data on the bottom and top.
    ``geom`` 'curvy_annulus' is the reference's third test (tests/test_2d.py:54-55)
    at a smaller size; 'square' is Helmholtz with Gaussian bumps on the unit
    square.  Both the reference's slabLU (cyclic interface solver) and its
    superLU path (folded sparse matrix) are recorded, with the partition."""
    nwaves = int(n / ppw)
    kh = (nwaves + 0.03) * 2 * np.pi + 1.8
    if geom == 'square':
        op = ref_pdo.PDO_2d(ref_pdo.ones, ref_pdo.ones,
                            c=lambda xx: bif.bfield_gaussian_bumps(xx, kh).reshape(-1))
        pmap = lambda xx: xx.clone()
    else:
        op, pmap, _ = ref_pdo.get_param_map_and_pdo(geom, bif.bfield_constant, kh)
    a = 1 / (2 * (n / (p - 2)))
    uu = lambda xx: bif.uu_dir_func_greens(pmap(xx), kh)
    out = dict(p=p, n=n, ppw=ppw, kh=kh, stride=stride, box=np.asarray(box))
    for solver in ('slabLU', 'superLU'):
        dom = Domain_Solver(torch.tensor(box), op, kh, a, p=p, buf_constant=1.0, periodic_bc=True)
        dom.build('reduced_cpu', solver, verbose=False)
        sol, res, tres, rloc, _ = dom.solve(uu, None, known_sol=True)
        sol, res, tres, rloc, _ = dom.solve(uu, None, known_sol=True)
        sol = sol.numpy()
        out.update({solver + '_sol_sub': sol[::stride], solver + '_sol_norm': np.linalg.norm(sol),
                    solver + '_res': float(res), solver + '_trueres': float(tres),
                    solver + '_resloc': float(rloc)})
    out.update(buf=np.array(dom.buf_pans), Npan=np.array(dom.Npan), nbox=dom.hps.n.numpy())
    for nm in ('I_Ctot', 'I_Xtot', 'I_slabX', 'I_Ctot_unique', 'I_Ctot_copy1', 'I_Ctot_copy2'):
        v = np.ascontiguousarray(np.asarray(getattr(dom, nm)), dtype=np.int64)
        if v.size <= 10000:
            out[nm] = v
        else:  # large index sets: length and SHA-256 of the int64 bytes
            out[nm + '_size'] = np.array(v.size)
            out[nm + '_sha256'] = np.array(hashlib.sha256(v.tobytes()).hexdigest())
    if geom != 'square':
        xx = dom.hps.xx_tot
        pick = np.arange(0, xx.shape[0], 397)
        xs = xx[pick]
        out.update(coef_xx=xs.numpy(), mapped_xx=pmap(xs).numpy())
        for k in ('c11', 'c22', 'c12', 'c1', 'c2', 'c'):
            f = getattr(op, k)
            out['coef_' + k] = np.zeros(xs.shape[0]) if f is None else np.asarray(f(xs)).reshape(-1)
    save(name, **out)


def hbs_kernel(x, j):
    """Test operator for HBS compression: a smooth, slowly decaying interaction plus a
    diagonal (numerically low-rank off-diagonal blocks, as the slab interface blocks)."""
    d = (x[:, None] - x[None, :]).abs()
    return (1.0 + 0.3 * j) / (1.0 + 40.0 * d) + (2.0 + j) * torch.eye(x.shape[0])


def hbs_fixture():
    """The reference's HBS compression from sketches (src_solver/hbs_reconstruction.py)
    on small test operators: the sketches, the compressed tensors, products with the
    compressed matrix and its transpose, and the compressed inverse."""
    from src_solver.hbs_reconstruction import HBS_matrix
    out = {}
    for tag, (b, n, k, seed) in (('L3', (2, 64, 4, 11)), ('L1', (2, 32, 8, 12)), ('pad', (1, 48, 4, 13))):
        torch.manual_seed(seed)
        x = torch.rand(n).sort().values
        A = torch.stack([hbs_kernel(x, j) for j in range(b)])
        hbs = HBS_matrix(b, n, k)
        ns = hbs.bs + k
        Om = torch.rand(1, n, ns)
        Ps = torch.rand(1, n, ns)
        Y = A @ Om
        Z = A.transpose(-1, -2) @ Ps
        state = torch.get_rng_state()
        hbs.reconstruct(Om.clone(), Ps.clone(), Y.clone(), Z.clone())
        if hbs.n_pad > 0:  # replay the padding sketches the reference drew inside reconstruct
            torch.set_rng_state(state)
            out[tag + '_Om_pad'] = torch.rand(1, hbs.n_pad, ns).numpy()
            out[tag + '_Ps_pad'] = torch.rand(1, hbs.n_pad, ns).numpy()
        q = torch.randn(b, n, 3)
        f = torch.randn(b, n, 2)
        out.update({tag + '_x': x.numpy(), tag + '_Om': Om.numpy(), tag + '_Ps': Ps.numpy(),
                    tag + '_Y': Y.numpy(), tag + '_Z': Z.numpy(),
                    tag + '_shape': np.array([b, n, k, hbs.bs, hbs.m, hbs.n_pad, hbs.L]),
                    tag + '_q': q.numpy(), tag + '_mv': hbs.matvec(q.clone()).numpy(),
                    tag + '_mvT': hbs.matvec(q.clone(), transpose=True).numpy()})
        if n <= 32:  # the compressed tensors (copies: calc_inverse updates D in place) and the dense matrix
            out.update({tag + '_UV': hbs.UVtensor.clone().numpy(), tag + '_D': hbs.Dtensor.clone().numpy(),
                        tag + '_dense': hbs.todense().numpy()})
        hbs.calc_inverse()
        out.update({tag + '_f': f.numpy(), tag + '_inv': hbs.apply_inverse(f.clone()).numpy(),
                    tag + '_invT': hbs.apply_inverse(f.clone(), transpose=True).numpy()})
    save('hbs.npz', **out)


def fd_fixture(name, n, ppw, pde, box=((0, 1.0), (0, 1.0)), buf_constant=0.6, stride=7):
    """The reference's finite-difference discretisation (src_disc/fd_disc.py,
    --disc fd in argparse_driver.py:144-150): the grid, its index sets, the
    five-point operator, the slab partition, and the superLU and slabLU
    solutions with free-space Dirichlet data."""
    nwaves = int(n / ppw)
    kh = (nwaves + 0.03) * 2 * np.pi + 1.8
    if pde == 'bfield_constant':
        cf = lambda xx: bif.bfield_constant(xx, kh)
    else:
        cf = lambda xx: bif.bfield_gaussian_bumps(xx, kh).reshape(-1)
    op = ref_pdo.PDO_2d(ref_pdo.ones, ref_pdo.ones, c=cf)
    h = 1 / n
    uu = lambda xx: bif.uu_dir_func_greens(xx, kh)
    out = dict(n=n, ppw=ppw, kh=kh, h=h, box=np.asarray(box), buf_constant=buf_constant, stride=stride)
    for solver in ('superLU', 'slabLU'):
        dom = Domain_Solver(torch.tensor(box), op, kh, h, buf_constant=buf_constant)
        dom.build('reduced_cpu', solver, verbose=False)
        sol, res, tres, rloc, _ = dom.solve(uu, None, known_sol=True)
        sol, res, tres, rloc, _ = dom.solve(uu, None, known_sol=True)
        sol = sol.numpy()
        out.update({solver + '_sol_sub': sol[::stride], solver + '_sol_norm': np.linalg.norm(sol),
                    solver + '_res': float(res), solver + '_trueres': float(tres)})
    fd = dom.fd
    A = dom.A.tocsr()
    A.sort_indices()
    out.update(ns=fd.ns.numpy(), XX=fd.XX.numpy()[::stride], buf=np.array(dom.buf), buf_prime=np.array(dom.buf_prime),
               Npan=np.array(dom.Npan), Npan_loc=np.array(dom.Npan_loc), A_data_sub=A.data[::stride],
               A_nnz=np.array(A.nnz), A_indptr_sha=np.array(hashlib.sha256(A.indptr.astype(np.int64).tobytes()).hexdigest()),
               A_indices_sha=np.array(hashlib.sha256(A.indices.astype(np.int64).tobytes()).hexdigest()))
    for nm in ('I_L', 'I_R', 'I_D', 'I_U', 'I_C', 'I_Ctot', 'I_Xtot'):
        out[nm] = np.asarray(getattr(dom, nm))
    out['I_X'] = np.asarray(fd.I_X)
    out['inds_pans'] = np.asarray(dom.inds_pans)
    save(name, **out)


def param_map_fixture(name='param_maps.npz', kh=25.0, seed=9):
    """The reference's parameter maps (src_disc/pdo.py:164-319) at seeded points of the
    unit square (and of [0, 6] x [0, 1] for the curvy annulus): mapped points and every
    coefficient of the pulled-back operator."""
    rng = np.random.default_rng(seed)
    out = {}
    for geom, xmax in (('curved', 1.0), ('annulus', 1.0), ('curvy_annulus', 6.0)):
        xs = torch.tensor(rng.random((200, 2)) * np.array([xmax, 1.0]))
        op, pmap, inv = ref_pdo.get_param_map_and_pdo(geom, bif.bfield_constant, kh)
        out[geom + '_xx'] = xs.numpy()
        out[geom + '_mapped'] = pmap(xs.clone()).numpy()
        for k in ('c11', 'c22', 'c12', 'c1', 'c2', 'c'):
            f = getattr(op, k)
            out[geom + '_' + k] = np.zeros(xs.shape[0]) if f is None else np.asarray(f(xs.clone())).reshape(-1)
    out['kh'] = np.array(kh)
    save(name, **out)


def solve_fixtures():
    dom, kh, sol, res, tres, rloc = run_domain(8, 48, 10, 'bfield_gaussian_bumps', 'superLU')
    save('solve_superlu_p8_n48.npz', p=8, n=48, kh=kh, sol=sol, res=res, trueres=tres, resloc=rloc)
    for (p, n, ppw, pde) in ((12, 400, 10, 'bfield_constant'), (22, 400, 40, 'bfield_constant')):
        dom, kh, sol, res, tres, rloc = run_domain(p, n, ppw, pde, 'slabLU')
        stride = 7
        save(f'slablu_p{p}_n{n}_ppw{ppw}.npz', p=p, n=n, ppw=ppw, kh=kh, stride=stride,
             sol_sub=sol[::stride], sol_norm=np.linalg.norm(sol), res=res, trueres=tres,
             resloc=rloc)



def _ref_threads():
    """Host threads for the reference runs: SLAB_REF_THREADS, default 1.  With more
    than one thread, batched torch.linalg.lu_factor / solve on the CPU (the torch
    2.11 + MKL 2024.2 build of this image) stops making progress on some hosts; one
    thread always completes."""
    return int(os.environ.get('SLAB_REF_THREADS', '1'))


def _product_problems():
    """The seeded synthetic fields of the benchmark configurations (the product's
    own generators, so that the fixture and the GPU runs see the same input)."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from slablu_gb300 import problems
    return problems


def _solve_config(cfg, solver, uu, extra_rhs=(), stride=331):
    """Reference Domain_Solver on the unit square for a problem dict of
    slablu_gb300.problems: build, then the driver's two solves (the second is the
    timed one, argparse_driver.py:169-170, 250-258), then the extra right-hand
    sides on the same factorization."""
    p, kh, a = cfg['p'], cfg['kh'], cfg['a']
    op = ref_pdo.PDO_2d(ref_pdo.ones, ref_pdo.ones, c=lambda xx: cfg['c'](xx).reshape(-1))
    t0 = time.time()
    dom = Domain_Solver(torch.tensor([[0, 1.0], [0, 1.0]]), op, kh, a, p=p, buf_constant=1.0)
    t_disc = time.time() - t0
    t0 = time.time()
    info = dom.build('reduced_cpu', solver, verbose=False)
    t_build = time.time() - t0
    dom.solve(uu, None, known_sol=False)
    t0 = time.time()
    sol, res, _, rloc, toc_solve = dom.solve(uu, None, known_sol=False)
    t_solve = time.time() - t0
    sol = sol.numpy()[:, 0]
    out = dict(stride=stride, sol_sub=sol[::stride], sol_norm=np.linalg.norm(sol), sol_len=sol.size,
               res=float(res), resloc=float(rloc), t_disc=t_disc, t_build=t_build, t_solve=t_solve,
               toc_build=float(info.get('toc_build', info.get('toc_build_blackbox', np.nan))),
               toc_assembly=float(info['toc_assembly']), toc_solve=float(toc_solve),
               threads=torch.get_num_threads())
    for k, col in enumerate(extra_rhs):
        f = lambda xx, col=col: torch.as_tensor(col).reshape(-1, 1) if xx.shape[0] == col.shape[0] else uu(xx)
        s2, r2, _, _, _ = dom.solve(f, None, known_sol=False)
        s2 = s2.numpy()[:, 0]
        out.update({f'rhs{k}_sol_sub': s2[::stride], f'rhs{k}_sol_norm': np.linalg.norm(s2), f'rhs{k}_res': float(r2)})
    return dom, out


def config3_fixture(solver='slabLU'):
    """Config 3 (p = 22, n = 2000, N = 4,404,000): the Gaussian-lattice Helmholtz
    field with Dirichlet data u = 1, solved by the reference itself (its slabLU,
    or its superLU black-box path); with slabLU also two of config 4's smoothed
    random boundary-data columns (0 and 255) on the same factorization."""
    problems = _product_problems()
    cfg = problems.config3()
    torch.set_num_threads(_ref_threads())
    uu = lambda xx: torch.ones(xx.shape[0], 1)
    # config 4's boundary data is defined on the Dirichlet nodes I_Xtot, in their order
    cfg_dom = Domain_Solver(torch.tensor([[0, 1.0], [0, 1.0]]), ref_pdo.PDO_2d(ref_pdo.ones, ref_pdo.ones), 0.0,
                            cfg['a'], p=cfg['p'], buf_constant=1.0)
    nbnd = len(cfg_dom.I_Xtot)
    del cfg_dom
    B = problems.config4_rhs(nbnd, 256).numpy()
    extra = (B[:, 0].copy(), B[:, 255].copy()) if solver == 'slabLU' else ()
    dom, out = _solve_config(cfg, solver, uu, extra)
    out.update(p=cfg['p'], n=cfg['n'], kh=cfg['kh'], nbnd=nbnd, rhs_cols=np.array([0, 255]), solver=solver,
               N=int((cfg['p'] - 2) * (cfg['p'] * dom.hps.n[0] * dom.hps.n[1] + dom.hps.n[0] + dom.hps.n[1])))
    print({k: v for k, v in out.items() if np.ndim(v) == 0})
    save(f'config3_{solver}_p22_n2000.npz', **out)


def config1_fixture():
    """Config 1 (p = 12, n = 400): constant-coefficient Helmholtz at 10 points per
    wavelength with Dirichlet data a sum of 8 seeded plane waves, solved by the
    reference's slabLU."""
    problems = _product_problems()
    cfg = problems.config1()
    torch.set_num_threads(_ref_threads())
    dom, out = _solve_config(cfg, 'slabLU', cfg['uu_dir'], stride=7)
    out.update(p=cfg['p'], n=cfg['n'], kh=cfg['kh'])
    print({k: v for k, v in out.items() if np.ndim(v) == 0})
    save('config1_slabLU_p12_n400.npz', **out)


def config2_fixture(picks=(0, 1, 127, 128, 5000, 8191, 8256, 12345, 16256, 16383)):
    """Config 2 (16,384 leaves of a 128 x 128 tiling, p = 22): the reference's
    form_DtNs in FP64 (hps_parallel_leaf_ops.py:40-72) on a sample of the leaves
    of the 32-bump field, c = -kh^2 b.  The leaf points follow the reference's
    get_grid (hps_multidomain_disc.py:111-124: leaf i*n1 + j is centred at
    (a + 2a i, a + 2a j)); the whole multidomain object is not built, its index
    bookkeeping for 16,384 leaves takes very long."""
    problems = _product_problems()
    cfg = problems.config2()
    p, a, kh, ns = cfg['p'], cfg['a'], cfg['kh'], cfg['nside']
    H = HPS_Disc(a, p, 2)
    Ds = torch.stack((torch.tensor(H.Ds.D11), torch.tensor(H.Ds.D22), torch.tensor(H.Ds.D12),
                      torch.tensor(H.Ds.D1), torch.tensor(H.Ds.D2)))
    zz = torch.tensor(H.zz.T)
    picks = list(picks)
    xx = torch.zeros(len(picks), p * p, 2)
    for t, box in enumerate(picks):
        i, j = divmod(box, ns)
        xx[t, :, 0] = zz[:, 0] + a + 2 * a * i
        xx[t, :, 1] = zz[:, 1] + a + 2 * a * j
    cvals = cfg['c'](xx.reshape(-1, 2)).reshape(-1)
    op = ref_pdo.PDO_2d(ref_pdo.ones, ref_pdo.ones, c=lambda x: cvals if x.shape[0] == cvals.shape[0] else None)
    DtN = leaf_ops.form_DtNs(p, 2, xx, torch.tensor(H.Nx), torch.tensor(H.JJ.Jx), torch.tensor(H.JJ.Jc),
                             torch.tensor(H.JJ.Jxreorder), Ds, torch.tensor(H.Interp_mat), op, 0, len(picks),
                             torch.device('cpu'), 'build', torch.zeros(len(picks), 4 * (p - 2), 1), None)
    save('config2_dtn_p22.npz', p=p, a=a, kh=kh, nside=ns, picks=np.asarray(picks), xx=xx.numpy(),
         c=cvals.reshape(len(picks), -1).numpy(), dtn=DtN.numpy())


if __name__ == '__main__':
    if len(sys.argv) > 2 and sys.argv[2] == 'config3':  # config 3 by the reference's slabLU (minutes)
        config3_fixture('slabLU')
        sys.exit(0)
    if len(sys.argv) > 2 and sys.argv[2] == 'config3_superlu':  # config 3 by its superLU (~11 min, 22 GB)
        config3_fixture('superLU')
        sys.exit(0)
    if len(sys.argv) > 2 and sys.argv[2] == 'configs':  # configs 1 and 2
        config1_fixture()
        config2_fixture()
        sys.exit(0)
    if len(sys.argv) > 2 and sys.argv[2] == 'maps':  # only the parameter-map fixture
        param_map_fixture()
        sys.exit(0)
    if len(sys.argv) > 2 and sys.argv[2] == 'fd':  # only the finite-difference fixture
        fd_fixture('fd_n120_ppw20.npz', 120, 20, 'bfield_constant')
        sys.exit(0)
    if len(sys.argv) > 2 and sys.argv[2] == 'hbs':  # only the HBS compression fixture
        hbs_fixture()
        sys.exit(0)
    if len(sys.argv) > 2 and sys.argv[2] == 'periodic_full':  # the reference's third test at its own size
        periodic_fixture('periodic_curvy_annulus_p22_n400.npz', 'curvy_annulus', [[0, 6.0], [0, 1.0]], 22, 400, 40,
                         stride=97)
        sys.exit(0)
    if len(sys.argv) > 2 and sys.argv[2] == 'periodic':  # only the periodic-boundary fixtures
        periodic_fixture('periodic_curvy_annulus_p12_n230.npz', 'curvy_annulus', [[0, 6.0], [0, 1.0]], 12, 230, 40,
                         stride=41)
        periodic_fixture('periodic_square_p12_n210.npz', 'square', [[0, 1.0], [0, 1.0]], 12, 210, 40, stride=7)
        sys.exit(0)
    if len(sys.argv) > 2 and sys.argv[2] == 'c12':  # only the mixed-derivative fixtures
        dtn_c12_fixture(12, 0.0125, 40, [0, 7, 800, 1599], 60.0, 'dtn_c12_p12.npz', seed=5)
        dtn_c12_fixture(8, 1 / 64, 32, [0, 5, 500, 1023], 40.0, 'dtn_c12_p8.npz', seed=6)
        annulus_fixture()
        sys.exit(0)
    leaf_fixtures()
    dtn_fixture(22, 0.005, 100, [0, 57, 4950, 9999, 1234, 6789, 3210, 8888], 1258.6, 'dtn_p22.npz')
    dtn_fixture(12, 0.0125, 40, [0, 7, 800, 1599], 253.3, 'dtn_p12.npz', seed=3)
    assembly_fixture()
    partition_fixture()
    blocktri_fixture()
    solve_fixtures()
