"""Fixed workloads for profiling single phases on one GPU.

    python -m slablu_gb300.profile_cases factor --n 640 --precision mixed
    python -m slablu_gb300.profile_cases solve  --n 2000 --precision mixed --iters 1
    python -m slablu_gb300.profile_cases dgemm  --n 2000 --reps 2
    python -m slablu_gb300.profile_cases sgemm  --n 4000 --k 200 --batch 10 --reps 2
    python -m slablu_gb300.profile_cases graph  --n 400 --count 8 --reps 3

`factor` and `solve` use the Gaussian-lattice Helmholtz field of the benchmark
(p = 22) on an n x n-point grid ((n/20)^2 leaves): one factorization, and for
`solve` one refined solve with at most --iters steps (u = 1 on the boundary, or
--nrhs columns of config 4's smoothed random boundary data).  `dgemm` runs --reps
tensor-core FP64 products C = A B of n x n random matrices (the shape of the
interface Schur update at n = 2000); `sgemm` runs --reps batched TF32-split FP32
products C -= A B with A n x k and B k x n (--batch of them: the shape of the
top merge level's Schur updates at N = 4.4M); `graph` factors --count engines of
alternating sizes (n and n/2 points a side) and times their refined solves
(u = 1 on the boundary, tol 1e-10) one after another through slab_engine_solve
against one launch of a SolveGraph over all of them.
"""
import argparse

import torch

from . import hps, problems
from .engine import SlabEngine


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument('case', choices=['factor', 'solve', 'dgemm', 'sgemm', 'graph'])
    ap.add_argument('--n', type=int, default=640)
    ap.add_argument('--precision', default='mixed', choices=['fp64', 'mixed', 'fp32'])
    ap.add_argument('--iters', type=int, default=1)
    ap.add_argument('--reps', type=int, default=2)
    ap.add_argument('--k', type=int, default=200)
    ap.add_argument('--batch', type=int, default=10)
    ap.add_argument('--count', type=int, default=8)
    ap.add_argument('--nrhs', type=int, default=1, help='solve: right-hand sides (config 4 data when > 1)')
    a = ap.parse_args(argv)
    if a.case == 'graph':
        return _graph_case(a)
    if a.case == 'sgemm':
        from .dgemm import sgemm_tc
        gen = torch.Generator(device='cuda').manual_seed(1)
        A = torch.randn(a.batch, a.n, a.k, dtype=torch.float32, device='cuda', generator=gen)
        B = torch.randn(a.batch, a.k, a.n, dtype=torch.float32, device='cuda', generator=gen)
        C = torch.zeros(a.batch, a.n, a.n, dtype=torch.float32, device='cuda')
        times = []
        for _ in range(a.reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            C = sgemm_tc(A, B, C, alpha=-1.0, beta=1.0)
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        print('ok sgemm', a.batch, a.n, a.k, float(C.abs().max()), 'ms per batch (incl. layout copies and slicing):',
              [round(t, 3) for t in times])
        return
    if a.case == 'dgemm':
        from .dgemm import dgemm_emu
        gen = torch.Generator(device='cuda').manual_seed(1)
        A = torch.randn(a.n, a.n, dtype=torch.float64, device='cuda', generator=gen)
        B = torch.randn(a.n, a.n, dtype=torch.float64, device='cuda', generator=gen)
        times = []
        for _ in range(a.reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            C = dgemm_emu(A, B)
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        print('ok dgemm', a.n, float(C.abs().max()), 'ms per product (incl. slicing):', [round(t, 3) for t in times],
              'FP64-equivalent TFLOP/s of the best:', round(2 * a.n ** 3 / (min(times) / 1e3) / 1e12, 2))
        return
    cfg = problems.config3()
    p = cfg['p']
    g = hps.Geometry([[0, 1], [0, 1]], problems.leaf_half_width(a.n, p), p, 1.0)
    xx = torch.as_tensor(g.xx_tot, device='cuda')
    c = cfg['c'](xx).contiguous()
    one = torch.ones_like(c)
    eng = SlabEngine(g, a.precision)
    eng.factor(c11=one, c22=one, c=c)
    if a.case == 'solve':
        if a.nrhs > 1:
            B = torch.zeros(g.ntot, a.nrhs, dtype=torch.float64, device='cuda')
            ix = torch.as_tensor(g.I_Xtot, device='cuda')
            B[ix] = problems.config4_rhs(len(g.I_Xtot), a.nrhs).to('cuda')
        else:
            B = torch.ones(g.ntot, dtype=torch.float64, device='cuda')
        _, _, it, info = eng.solve(B, tol=1e-10, max_iter=a.iters, allow_noconv=True)
        print('refinement steps', it, info)
    torch.cuda.synchronize()
    print('ok', a.case, g.nboxes, 'leaves', eng.timings())


def _graph_case(a):
    from .engine import SolveGraph
    cfg = problems.config3()
    p = cfg['p']
    engines, bnds = [], []
    for i in range(a.count):
        n = a.n if i % 2 == 0 else max(20, (a.n // 40) * 20)
        g = hps.Geometry([[0, 1], [0, 1]], problems.leaf_half_width(n, p), p, 1.0)
        c = cfg['c'](torch.as_tensor(g.xx_tot, device='cuda')).contiguous()
        eng = SlabEngine(g, a.precision)
        eng.factor(c11=torch.ones_like(c), c22=torch.ones_like(c), c=c)
        engines.append(eng)
        bnds.append(torch.ones(g.ntot, dtype=torch.float64, device='cuda'))
    graph = SolveGraph(engines, nrhs=1, tol=1e-10, max_iter=40)
    for i, b in enumerate(bnds):
        graph.set_inputs(i, b)

    def timed(fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)
    seq, one = [], []
    for _ in range(a.reps + 1):
        seq.append(timed(lambda: [e.solve(b, tol=1e-10, max_iter=40) for e, b in zip(engines, bnds)]))
        one.append(timed(lambda: (graph.launch(), [graph.result(i) for i in range(len(engines))])))
    its = [graph.result(i)[1] for i in range(len(engines))]
    err = max(float(torch.linalg.norm(graph.result(i)[0][:, 0] - e.solve(b, tol=1e-10, max_iter=40)[0][:, 0]) /
                    torch.linalg.norm(graph.result(i)[0]))
              for i, (e, b) in enumerate(zip(engines, bnds)))
    print('ok graph', a.count, 'engines', [e.nleaf for e in engines], 'leaves; steps', its,
          '; ms one after another', [round(t, 3) for t in seq[1:]], '; ms one graph', [round(t, 3) for t in one[1:]],
          '; max rel difference', err)


if __name__ == '__main__':
    main()
