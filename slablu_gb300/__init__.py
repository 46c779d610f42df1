"""slablu_gb300: GB300-native SlabLU factor-and-solve path (HPS discretisation
of a rectangle; curved domains through the reference's parameter maps).

Public API mirrors the reference (annayesy/slabLU):
    Domain_Solver(box_geom, pdo_op, kh, a, p=..., buf_constant=..., periodic_bc=...)
        .build(sparse_assembly='reduced_gpu', solver_type='slabLU')
        .solve(uu_dir_func, ff_body_func=None, known_sol=False)
    pdo.get_param_map_and_pdo(geom, bfield, kh)
plus SlabEngine / leaf_dtn for direct use of the C ABI (include/slablu_gb300.h)
and slab_solve, a torch.autograd.Function over factor + solve whose backward
is the hand-written adjoint.
"""
import torch

torch.set_default_dtype(torch.double)  # the reference's modules set this on import

from . import pdo, built_in_funcs, hps  # noqa: E402,F401
from .engine import SlabEngine, SolveGraph, leaf_dtn  # noqa: E402,F401
from .slablu_solver import Domain_Solver  # noqa: E402,F401
from .adjoint import slab_solve  # noqa: E402,F401

__all__ = ['Domain_Solver', 'SlabEngine', 'SolveGraph', 'leaf_dtn', 'slab_solve', 'pdo', 'built_in_funcs', 'hps']
