"""Differentiable factor-and-solve: a torch.autograd.Function over the engine.

Forward: factor A(c) with the given coefficient fields and solve A u = f with
Dirichlet data (slab_engine_factor / slab_engine_solve).  Backward: one
transposed solve with the stored factors (slab_engine_adjoint) and the
coefficient-gradient kernel (slab_engine_coeff_grad; slab_engine_coeff_grad_mixed
for an engine with a mixed derivative c12, whose gradient it also gives).  The
reference has no adjoint; its transposed building blocks are
lusolve_sweep_transpose (src_solver/block_tridiag_solver_dense.py:205-222) and
solve_slab(transpose=True) (src_solver/slablu_solver.py:901-943).

    eng = SlabEngine(geom, 'mixed')
    b = torch.tensor(..., requires_grad=True)           # field at the leaf nodes
    c = -kh**2 * (1 - b)                                 # any torch expression
    u = slab_solve(eng, bnd, c=c, c11=ones, c22=ones)    # (npts, nrhs)
    loss = (w * u).sum(); loss.backward()                # b.grad = dL/db
"""
import torch

from .engine import SlabEngine

_KEYS = ('c11', 'c22', 'c12', 'c1', 'c2', 'c')


class _SlabSolve(torch.autograd.Function):

    @staticmethod
    def forward(ctx, engine, keys, tol, max_iter, bnd, fbody, *coefs):
        engine.factor(**dict(zip(keys, [c.detach().reshape(-1).contiguous() for c in coefs])))
        uleaf, ufaces, iters, info = engine.solve(bnd.detach(), None if fbody is None else fbody.detach(), tol=tol,
                                                  max_iter=max_iter, want_faces=True)
        ctx.engine, ctx.keys, ctx.tol, ctx.max_iter = engine, keys, tol, max_iter
        ctx.generation = engine.generation
        ctx.bnd_dim, ctx.coef_shapes = bnd.dim(), [c.shape for c in coefs]
        ctx.has_fbody = fbody is not None
        ctx.fbody_dim = None if fbody is None else fbody.dim()
        ctx.save_for_backward(uleaf, ufaces)
        ctx.info = dict(iters=iters, **info)
        return uleaf if bnd.dim() > 1 else uleaf[:, 0]

    @staticmethod
    def backward(ctx, g):
        engine = ctx.engine
        if engine.generation != ctx.generation:
            raise RuntimeError('slab_solve: the engine was refactored between forward and backward')
        uleaf, ufaces = ctx.saved_tensors
        g = g.reshape(uleaf.shape).to(torch.float64)
        lam, _, gbnd, iters, info = engine.adjoint(gleaf=g, tol=ctx.tol, max_iter=ctx.max_iter, want_bnd=True)
        need = [k for k, n in zip(ctx.keys, ctx.needs_input_grad[6:]) if n]
        grads = engine.coeff_grad(ufaces, uleaf, lam, keys=tuple(need)) if need else {}
        coef_grads = [grads[k].reshape(shp) if k in grads else None for k, shp in zip(ctx.keys, ctx.coef_shapes)]
        gb = None
        if ctx.needs_input_grad[4]:
            gb = gbnd if ctx.bnd_dim > 1 else gbnd[:, 0]
        gf = None
        if ctx.has_fbody and ctx.needs_input_grad[5]:
            gf = lam if ctx.fbody_dim > 1 else lam[:, 0]
        return (None, None, None, None, gb, gf, *coef_grads)


def slab_solve(engine: SlabEngine, bnd, fbody=None, tol=1e-12, max_iter=30, **coeffs):
    """Solve A(c) u = f on the engine's geometry, differentiable in the
    coefficient fields (each a (npts,) float64 CUDA tensor), the Dirichlet data
    bnd ((ntot,) or (ntot, nrhs)) and the body load fbody ((npts,) or (npts, nrhs)).
    Returns u at every leaf node, (npts,) or (npts, nrhs)."""
    keys = tuple(k for k in _KEYS if coeffs.get(k) is not None)
    unknown = set(coeffs) - set(_KEYS)
    if unknown:
        raise ValueError(f'unknown coefficients {sorted(unknown)}')
    coefs = [coeffs[k].to(torch.float64) for k in keys]
    return _SlabSolve.apply(engine, keys, tol, max_iter, bnd.to(torch.float64),
                            None if fbody is None else fbody.to(torch.float64), *coefs)


def fd_check(loss_fn, b, v, ad, steps=(1e-5, 1e-6, 1e-7)):
    """Central differences of loss_fn along v with the step chosen a posteriori:
    for each h the estimates at h and h/2 are combined by Richardson extrapolation
    (the O(h^2) term cancels) and their discrepancy |fd(h) - fd(h/2)| estimates the
    error; the step with the smallest estimate is kept.  The adjoint value ad is
    used only for the reported error, not for the choice.  Returns
    (relative error against ad, chosen step, error estimate)."""
    best = None
    for h in steps:
        fd = []
        for hh in (h, h / 2):
            fd.append((float(loss_fn(b + hh * v)) - float(loss_fn(b - hh * v))) / (2 * hh))
        rich = (4 * fd[1] - fd[0]) / 3
        est = abs(fd[1] - fd[0]) / max(abs(rich), 1e-300)
        if best is None or est < best[2]:
            best = (rich, h, est)
    rich, h, est = best
    return abs(rich - ad) / max(abs(rich), 1e-300), h, est
