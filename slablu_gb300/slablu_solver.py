"""Drop-in ``Domain_Solver`` for the HPS SlabLU factor-and-solve path on one GPU.

Mirrors src_solver/slablu_solver.py:59-666 (constructor, ``build``,
``solve`` and the attributes its driver reads) for the unit-square HPS
discretisation with solver_type='slabLU'.  All factor and solve arithmetic runs
in libslablu_gb300.so (include/slablu_gb300.h); there is no CPU path.

Differences from the reference, by design:
  * ``sparse_assembly`` 'reduced_gpu' / 'reduced_gb300' select this GPU path;
    'reduced_cpu' raises (no CPU implementation is shipped).
  * the slab interface operators are formed exactly and densely instead of by
    randomised HBS compression (slablu_solver.py:1139-1308);
  * ``precision`` selects FP64, mixed (FP32 leaf and slab factors, FP64
    interface) or FP32 factors; every solve is refined against the FP64
    residual of the full HPS collocation system until the relative correction
    is below ``tol``.
  * ``rel_err`` returned by ``solve`` is that FP64 relative residual (the
    reference reports the residual of its reduced sparse system).
  * the reduced sparse operator is not needed by the solver; ``hps.sparse_mat``
    and ``get_rhs`` assemble and apply it on the GPU for callers of the
    reference's sparse interface (slablu_gb300/sparse.py).
  * periodic_bc=True couples the shared edge back through its Schur complement
    on top of the non-periodic factorization (slablu_gb300/periodic.py; the
    complement is LU-factored by the library's FP64 kernels) instead of the
    reference's cyclic interface solver; ``rel_err`` is then the relative
    residual of the folded reduced system, as in the reference.
  * a mixed derivative (c12, curved domains through a parameter map) runs
    the reference's c12 leaf branch (slab_engine_create_mixed); its adjoint
    is not provided.
Out of scope (raise NotImplementedError): finite differences (p = 0), body
loads with periodic_bc.
"""
import time
import warnings

import numpy as np
import torch

from . import _lib, periodic, sparse
from .engine import SlabEngine
from .hps import Geometry


class _HPSView:
    """The subset of HPS_Multidomain the reference driver reads (n, xx_tot,
    xx_active), and its reduced sparse operator (sparse_mat)."""

    def __init__(self, geom, coeff_fn=None):
        self.geom = geom
        self._coeff_fn = coeff_fn
        self.p, self.a = geom.p, geom.a
        self.n = torch.tensor([geom.n0, geom.n1], dtype=torch.int32)
        self.nboxes = geom.nboxes
        self.xx_tot = torch.as_tensor(geom.xx_tot)
        self.xx_active = torch.as_tensor(geom.xx_active)
        self.grid_xx = torch.as_tensor(geom.xx)

    def sparse_mat(self, device='cuda', verbose=False):
        """Reduced operator: leaf DtN maps (FP64, slab_leaf_dtn) summed on the GPU
        (hps_multidomain_disc.py:53-109).  Returns (A as a torch sparse CSR tensor on
        ``device``, timing dict), like the reference's (scipy CSR, t_dict)."""
        from . import sparse
        from .engine import leaf_dtn
        dev = torch.device(device)
        if dev.type != 'cuda':
            raise ValueError('sparse_mat is assembled on the GPU (device must be cuda)')
        if self._coeff_fn is None:
            raise RuntimeError('this view has no coefficients (use Domain_Solver.hps)')
        g = self.geom
        torch.cuda.synchronize()
        tic = time.time()
        co = {k: (None if v is None else v.reshape(g.nboxes, g.p * g.p)) for k, v in self._coeff_fn().items()}
        kw = {}
        if co.get('c12') is not None:  # mixed derivative: the Jxreorder / Interp_mat branch
            kw = dict(interp=g.ops.Interp_mat, jxreorder=g.ops.Jxreorder)
        dtn, info = leaf_dtn(co, g.p, g.ops.D, g.ops.Dsq, g.ops.Nx, precision='fp64', **kw)
        if int(info.abs().sum()) != 0:
            raise RuntimeError('leaf DtN: zero pivot in a leaf interior block')
        torch.cuda.synchronize()
        toc_dtn = time.time() - tic
        tic = time.time()
        A = sparse.assemble(g, dtn)
        torch.cuda.synchronize()
        t = dict(toc_DtN=toc_dtn, toc_forloop=0.0, toc_sparse=time.time() - tic)
        if verbose:
            print(f'\t--time to assemble sparse HPS (DtN ops, csr on the GPU) ({toc_dtn:5.2f},{t["toc_sparse"]:5.2f})')
        self._A = A
        return A.to_torch(), t


class Domain_Solver:
    def __init__(self, box_geom, pdo_op, kh, h, p=0, buf_constant=0.5, periodic_bc=False, precision='mixed',
                 tol=1e-10, max_iter=12, device='cuda'):
        if p == 0:
            raise NotImplementedError('slablu_gb300 provides the HPS discretisation only (p > 0)')
        self.kh = kh
        self.pdo = pdo_op
        self.buf_constant = buf_constant
        self.periodic_bc = bool(periodic_bc)
        # a mixed derivative (curved domains): the c12 branch of the leaf operators
        self.mixed = getattr(pdo_op, 'c12', None) is not None
        self.precision, self.tol, self.max_iter = precision, tol, max_iter
        self.device = torch.device(device)
        bg = box_geom.detach().cpu().numpy() if isinstance(box_geom, torch.Tensor) else np.asarray(box_geom)
        self.geom = Geometry(bg, h, p, buf_constant)
        g = self.geom
        self.disc = 'hps'
        self.hps = _HPSView(g, self._coeffs)
        self.buf_pans, self.Npan, self.Npan_loc = g.buf, g.Npan, g.n1
        self.ntot = g.ntot
        lt = lambda a: torch.as_tensor(a, dtype=torch.long)
        self.inds_pans = lt(g.inds_pans)
        self.I_L, self.I_R, self.I_D, self.I_U, self.I_C = (lt(g.I_L), lt(g.I_R), lt(g.I_D), lt(g.I_U), lt(g.I_C))
        self.I_slabC, self.I_slabX = lt(g.I_slabC), lt(g.I_slabX)
        self.I_Ctot, self.I_Xtot = lt(g.I_Ctot), lt(g.I_Xtot)
        if self.periodic_bc:
            self._psets = periodic.periodic_index_sets(g)
            ps = self._psets
            self.I_slabX, self.I_Ctot, self.I_Xtot = lt(ps['I_slabX']), lt(ps['I_Ctot']), lt(ps['I_Xtot'])
            self.I_Ctot_unique = lt(ps['I_Ctot_unique'])
            self.I_Ctot_copy1, self.I_Ctot_copy2 = lt(ps['I_Ctot_copy1']), lt(ps['I_Ctot_copy2'])
        self.engine = None
        self._edge = None
        self.solver_type = None

    # -- coefficients at every leaf node, evaluated on the device -----------------
    def _coeffs(self):
        # the leaf nodes go to the device on every build (from a pinned host copy)
        if getattr(self, '_xx_host', None) is None:
            self._xx_host = torch.as_tensor(self.geom.xx_tot, dtype=torch.float64)
            if self.device.type == 'cuda':
                self._xx_host = self._xx_host.pin_memory()
        xx = self._xx_host.to(self.device, non_blocking=True)
        out = {}
        for key in ('c11', 'c22', 'c1', 'c2', 'c') + (('c12',) if self.mixed else ()):
            f = getattr(self.pdo, key, None)
            if f is None:
                out[key] = None
                continue
            v = f(xx)
            v = torch.as_tensor(v, dtype=torch.float64).to(self.device).reshape(-1)
            if v.numel() != xx.shape[0]:
                raise ValueError(f'coefficient {key} returned {v.numel()} values for {xx.shape[0]} points')
            out[key] = v.contiguous()
        return out

    def build(self, sparse_assembly='reduced_gpu', solver_type='slabLU', verbose=True):
        """Factor the operator (slablu_solver.py:440-487).  Returns the build info dict."""
        if solver_type != 'slabLU':
            raise ValueError(f"solver_type {solver_type!r}: slablu_gb300 provides 'slabLU' only")
        if sparse_assembly not in ('reduced_gpu', 'reduced_gb300'):
            raise ValueError(f'sparse_assembly {sparse_assembly!r}: only the GPU path is provided')
        self.sparse_assembly, self.solver_type = sparse_assembly, solver_type
        torch.cuda.synchronize()
        tic = time.time()
        if self.engine is None:
            self.engine = SlabEngine(self.geom, self.precision, mixed=self.mixed)
        co = self._coeffs()
        torch.cuda.synchronize()
        toc_coeff = time.time() - tic
        tic2 = time.time()
        self.engine.factor(**co)
        torch.cuda.synchronize()
        toc_factor = time.time() - tic2
        toc_edge = 0.0
        if self.periodic_bc:
            tic3 = time.time()
            self._build_periodic_edge()
            torch.cuda.synchronize()
            toc_edge = time.time() - tic3
        toc_build = time.time() - tic
        info = dict(toc_build=toc_build, toc_assembly=toc_coeff, toc_factor=toc_factor,
                    mem_build=self.engine.factor_bytes / 1e9, precision=self.precision)
        if self.periodic_bc:
            info.update(toc_periodic_edge=toc_edge, periodic_edge_size=self._edge.nL)
        if verbose:
            print(f'SLABLU GB300 BUILD ({self.precision}): {toc_build:.3f} s, factors {info["mem_build"]:.2f} GB, '
                  f'buf={self.buf_pans} Npan={self.Npan}')
        return info

    def get_rhs(self, uu_dir_func, ff_body_func=None, sum_body_load=True):
        """Right-hand side of the reduced system on I_Ctot, ff = -A[I_Ctot, I_Xtot] uu_dir
        (slablu_solver.py:489-507), with A assembled on the GPU; a device tensor
        (len(I_Ctot), nrhs).  Body loads enter through solve(ff_body_func=...) instead:
        the reference's reduction of a body load to the faces (reduce_body,
        hps_parallel_leaf_ops.py:94-100) does not run."""
        if ff_body_func is not None:
            raise NotImplementedError('body loads: pass ff_body_func to solve()')
        if getattr(self.hps, '_A', None) is None:
            self.hps.sparse_mat(self.device)
        A = self.hps._A
        XX = self.hps.xx_active
        ud = torch.as_tensor(uu_dir_func(XX[self.I_Xtot]), dtype=torch.float64)
        if ud.dim() == 1:
            ud = ud[:, None]
        x = torch.zeros(self.ntot, ud.shape[1], dtype=torch.float64, device=self.device)
        x[self.I_Xtot.to(self.device)] = ud.to(self.device)
        ff = -A.matvec(x)[self.I_Ctot.to(self.device)]
        if self.periodic_bc and sum_body_load:
            ff = periodic.fold(ff, self._psets)
        return ff

    def _build_periodic_edge(self):
        """Schur complement of the shared edge (slablu_gb300/periodic.py), with the
        edge rows of the reduced operator assembled on the GPU."""
        g = self.geom
        if getattr(self.hps, '_A', None) is None:
            self.hps.sparse_mat(self.device)
        left, right = periodic.edge_faces(g)
        E = sparse.row_subset(g, self.hps._A, np.concatenate((left, right)))
        self._edge = periodic.PeriodicEdge(self.engine, E.matvec, left, right, self.ntot, tol=self.tol,
                                           max_iter=self.max_iter, dense_lu=periodic.DenseLU).build(self.device)

    def get_rhs_boundary(self, uu_dir_func):
        """Face vector carrying Dirichlet data at I_Xtot (slablu_solver.py:504)."""
        XX = self.hps.xx_active
        ud = torch.as_tensor(uu_dir_func(XX[self.I_Xtot]), dtype=torch.float64)
        if ud.dim() == 1:
            ud = ud[:, None]
        bnd = torch.zeros(self.ntot, ud.shape[1], dtype=torch.float64, device=self.device)
        bnd[self.I_Xtot.to(self.device)] = ud.to(self.device)
        return bnd

    def solve(self, uu_dir_func, ff_body_func=None, known_sol=False):
        """Solve and recover every leaf node (slablu_solver.py:623-666).

        Returns (sol_tot (N_leafnodes, nrhs) CPU tensor, rel_err, true_err, resloc_hps, toc_solve).
        """
        if self.engine is None:
            raise RuntimeError('call build() before solve()')
        torch.cuda.synchronize()
        tic = time.time()
        bnd = self.get_rhs_boundary(uu_dir_func)
        fb = None
        if ff_body_func is not None:
            if self.periodic_bc:
                raise NotImplementedError('body loads with periodic_bc are not provided')
            xx = torch.as_tensor(self.geom.xx_tot, dtype=torch.float64, device=self.device)
            fb = torch.as_tensor(ff_body_func(xx), dtype=torch.float64).to(self.device)
            if fb.dim() == 1:
                fb = fb[:, None]
        if self.periodic_bc:
            uleaf, uf, st = self._edge.solve(bnd)
            iters = st['engine_iters']
            rel_err = torch.tensor(self._folded_residual(uf, bnd))
        else:
            uleaf, _, iters, st = self.engine.solve(bnd, fb, tol=self.tol, max_iter=self.max_iter,
                                                    allow_noconv=True)
            rel_err = torch.tensor(st['rel_residual'])
            if not st['converged']:
                # the answer is still returned (with its residual, as the reference returns
                # rel_err), but it is less accurate than tol asks
                warnings.warn(f'refinement stopped after {iters} steps at relative correction '
                              f'{st["rel_correction"]:.1e} (tol {self.tol:.0e}): raise max_iter, or use '
                              f"precision='fp64' for a harder problem", RuntimeWarning, stacklevel=2)
        # the leaf-node solution comes back into pinned host memory (torch's
        # caching host allocator reuses the blocks of freed results)
        if uleaf.is_cuda:
            sol_tot = torch.empty(uleaf.shape, dtype=uleaf.dtype, pin_memory=True)
            sol_tot.copy_(uleaf)
        else:
            sol_tot = uleaf.cpu()
        toc_solve = time.time() - tic
        self.last_solve_info = dict(st, iters=iters)
        true_err = torch.tensor([float('nan')])
        if known_sol:
            uu_true = torch.as_tensor(uu_dir_func(self.hps.xx_tot.clone()), dtype=torch.float64)
            if uu_true.dim() == 1:
                uu_true = uu_true[:, None]
            true_err = torch.linalg.norm(sol_tot - uu_true) / torch.linalg.norm(uu_true)
        return sol_tot, rel_err, true_err, st['resloc'], toc_solve

    def _folded_residual(self, uf, bnd):
        """||A_CC x - ff|| / ||ff|| of the folded periodic reduced system
        (slablu_solver.py:528-541, 594-596), with A applied on the GPU: at the
        unknown faces, A u (u with the Dirichlet data) is A_CC x + A_CX d =
        A_CC x - ff, and -A d is ff."""
        A = self.hps._A
        bnd = bnd if bnd.dim() == 2 else bnd[:, None]
        d = torch.zeros_like(uf)
        ix = self.I_Xtot.to(uf.device)
        d[ix] = bnd[ix]
        ic = self.I_Ctot.to(uf.device)
        r = periodic.fold(A.matvec(uf)[ic], self._psets)
        ff = periodic.fold(-A.matvec(d)[ic], self._psets)
        fn = float(torch.linalg.norm(ff))
        return float(torch.linalg.norm(r)) / fn if fn > 0 else float(torch.linalg.norm(r))
