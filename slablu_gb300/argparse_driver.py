"""Command-line driver with the reference's flags (argparse_driver.py:17-38).

    python -m slablu_gb300.argparse_driver --disc hps --p 22 --n 1000 --ppw 10 \\
        --domain square --pde bfield_constant --bc free_space --solver slabLU

Builds once and solves twice (the second solve is the reported one), and
pickles ``build_info`` then ``solve_info`` with the reference's keys
(argparse_driver.py:169-188, 248-298).  Added flags: --precision, --tol.
--periodic_bc identifies the left and right edges of the box (Dirichlet data on
the bottom and top only), and --domain curved / annulus / curvy_annulus solve on
the image of the box under the reference's parameter maps (boundary data at the
mapped points), as in the reference (its tests run square, annulus, and
curvy_annulus with --box_xlim 6 --periodic_bc).  Out of scope here: --disc fd,
the superLU/PETSc black-box solvers, --disable_cuda (slablu_gb300 has no CPU
path).
"""
import argparse
import pickle

import numpy as np
import torch

from . import built_in_funcs, pdo
from .slablu_solver import Domain_Solver


def parse(argv=None):
    ap = argparse.ArgumentParser('Call direct solver for 2D domain.')
    ap.add_argument('--disc', type=str, required=True)
    ap.add_argument('--p', type=int, required=False)
    ap.add_argument('--n', type=int, required=True)
    ap.add_argument('--pde', type=str, required=True)
    ap.add_argument('--domain', type=str, required=True)
    ap.add_argument('--box_xlim', type=float, default=1.0)
    ap.add_argument('--box_ylim', type=float, default=1.0)
    ap.add_argument('--bc', type=str, required=True)
    ap.add_argument('--ppw', type=int, required=False)
    ap.add_argument('--nwaves', type=float, required=False)
    ap.add_argument('--solver', type=str, default='slabLU')
    ap.add_argument('--sparse_assembly', type=str, default='reduced_gpu')
    ap.add_argument('--pickle', type=str, required=False)
    ap.add_argument('--store_sol', action='store_true')
    ap.add_argument('--disable_cuda', action='store_true')
    ap.add_argument('--buf_constant', type=float, required=False)
    ap.add_argument('--periodic_bc', action='store_true')
    ap.add_argument('--precision', type=str, default='mixed', choices=['fp64', 'mixed', 'fp32'])
    ap.add_argument('--tol', type=float, default=1e-10)
    return ap.parse_args(argv)


def main(argv=None):
    args = parse(argv)
    if args.disc != 'hps':
        raise ValueError('slablu_gb300 provides the HPS discretisation only')
    if args.domain not in ('square', 'curved', 'annulus', 'curvy_annulus'):
        raise ValueError(f'unknown domain {args.domain}')
    if args.disable_cuda:
        raise ValueError('slablu_gb300 runs on the GPU only (no CPU path)')
    if args.p is None:
        raise ValueError('HPS selected but p not provided')
    n = args.n
    box_geom = torch.tensor([[0, args.box_xlim], [0, args.box_ylim]])
    if args.pde == 'poisson':
        if args.ppw is not None:
            raise ValueError
        op = pdo.PDO_2d(pdo.ones, pdo.ones)
        kh = 0
    elif args.pde.startswith('bfield'):
        if (args.ppw is None) == (args.nwaves is None):
            raise ValueError('set exactly one of ppw and nwaves for an oscillatory bfield')
        nwaves = int(n / args.ppw) if args.ppw is not None else args.nwaves
        kh = (nwaves + 0.03) * 2 * np.pi + 1.8
        if args.pde not in built_in_funcs.BFIELDS:
            raise ValueError(f'unknown pde {args.pde}')
        bfield = built_in_funcs.BFIELDS[args.pde]
        if args.domain == 'square':
            op = pdo.PDO_2d(pdo.ones, pdo.ones, c=lambda xx: bfield(xx, kh))
        else:  # a curved domain through its parameter map (argparse_driver.py:119-136)
            op, param_map, _ = pdo.get_param_map_and_pdo(args.domain, bfield, kh)
    else:
        raise ValueError(f'unknown pde {args.pde}')
    if args.domain != 'square' and not args.pde.startswith('bfield'):
        raise ValueError('curved domains are set up for the bfield operators')
    mapped = (lambda xx: param_map(xx)) if args.domain != 'square' else (lambda xx: xx)
    p = args.p
    buf_constant = 1.0 if args.buf_constant is None else args.buf_constant
    a = 1 / (2 * (n / (p - 2)))
    dom = Domain_Solver(box_geom, op, kh, a, p=p, buf_constant=buf_constant, periodic_bc=args.periodic_bc,
                        precision=args.precision, tol=args.tol)
    N = (p - 2) * (p * dom.hps.n[0] * dom.hps.n[1] + dom.hps.n[0] + dom.hps.n[1])
    build_info = dom.build(sparse_assembly=args.sparse_assembly, solver_type=args.solver, verbose=True)
    build_info.update(N=int(N), n=n, disc='hps', buf=dom.buf_pans * (p - 2), pde=args.pde, bc=args.bc,
                      domain=args.domain, solver=args.solver, sparse_assembly=args.sparse_assembly,
                      box_geom=box_geom, kh=kh, periodic_bc=args.periodic_bc, a=a, p=p)
    if args.bc == 'free_space':
        if args.pde != 'bfield_constant':
            raise ValueError('free_space data is the exact solution only for bfield_constant')
        uu_dir, known = (lambda xx: built_in_funcs.uu_dir_func_greens(mapped(xx), kh)), True
    elif args.bc == 'pulse':
        uu_dir, known = (lambda xx: built_in_funcs.uu_dir_pulse(mapped(xx), kh)), False
    elif args.bc == 'ones':
        uu_dir, known = (lambda xx: torch.ones(xx.shape[0], 1)), False
    elif args.bc == 'log_dist' and args.pde == 'poisson':
        uu_dir, known = (lambda xx: built_in_funcs.uu_dir_func_greens(xx, 0)), True
    else:
        raise ValueError(f'boundary condition {args.bc} is not provided')
    dom.solve(uu_dir, None, known_sol=known)
    sol, res, true_res, resloc, toc = dom.solve(uu_dir, None, known_sol=known)
    print('\t--Slab solver solved Ax=b residual %5.2e with known solution residual %5.2e and resloc_HPS %5.2e '
          'in time %5.2f s' % (float(res), float(true_res), float(resloc), toc))
    solve_info = dict(res_solve=res, trueres_solve=true_res, resloc_hps_solve=resloc, toc_solve=toc,
                      refine_iters=dom.last_solve_info['iters'], precision=args.precision,
                      unknowns_per_s=float(N) / (build_info['toc_build'] + toc))
    if args.store_sol:
        solve_info['xx'] = dom.hps.xx_tot
        solve_info['sol'] = sol
    if args.pickle is not None:
        with open(args.pickle, 'wb+') as f:
            pickle.dump(build_info, f)
            pickle.dump(solve_info, f)
    return build_info, solve_info


if __name__ == '__main__':
    main()
