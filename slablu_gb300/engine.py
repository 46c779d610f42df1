"""Python handle on the C-ABI factor-and-solve engine.

Thin ownership wrapper: device arrays are torch tensors (allocation and
streams only); all arithmetic runs in libslablu_gb300.so.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .hps import Geometry


def _col_major(x, rows):
    """(rows,) or (rows, k) tensor -> storage laid out column-major (k, rows)."""
    if x.dim() == 1:
        x = x[:, None]
    assert x.shape[0] == rows
    return x.T.contiguous()


class SlabEngine:
    """Factorization of the HPS operator on a ``Geometry`` (see include/slablu_gb300.h)."""

    def __init__(self, geom: Geometry, precision='mixed', stream=None, mixed=False):
        """mixed: the operator has a mixed derivative c12 (slab_engine_create_mixed);
        factor() then takes c12."""
        if precision not in _lib.PREC:
            raise ValueError(f'precision must be one of {sorted(_lib.PREC)}')
        if not torch.cuda.is_available():
            raise RuntimeError('slablu_gb300 needs a CUDA GPU (there is no CPU path)')
        self.L = _lib.lib()
        self.geom, self.precision = geom, precision
        self.stream = stream if stream is not None else torch.cuda.current_stream()
        ops = geom.ops
        h = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        self._host = dict(D=h(ops.D), Dsq=h(ops.Dsq), Nx=h(ops.Nx), interp=h(ops.Interp_mat),
                          jxr=np.ascontiguousarray(ops.Jxreorder, dtype=np.int32))
        handle = ctypes.c_void_p()
        self.mixed = bool(mixed)
        create = self.L.slab_engine_create_mixed if self.mixed else self.L.slab_engine_create
        st = create(ctypes.byref(handle), geom.p, geom.n0, geom.n1, geom.buf,
                                       _lib.PREC[precision],
                                       _lib.np_ptr(self._host['D'], ctypes.c_double),
                                       _lib.np_ptr(self._host['Dsq'], ctypes.c_double),
                                       _lib.np_ptr(self._host['Nx'], ctypes.c_double),
                                       _lib.np_ptr(self._host['interp'], ctypes.c_double),
                                       _lib.np_ptr(self._host['jxr'], ctypes.c_int),
                                       ctypes.c_void_p(self.stream.cuda_stream))
        _lib.check(st, 'slab_engine_create')
        self.h = handle
        self.ntot = int(self.L.slab_engine_nfaces(self.h))
        self.nleaf = int(self.L.slab_engine_nleaves(self.h))
        self.npts = self.nleaf * geom.p * geom.p
        self.n_int = (geom.p - 2) ** 2
        self.generation = 0  # incremented by every factor(); checked by the autograd backward

    def __del__(self):
        h = getattr(self, 'h', None)
        if h is not None and h.value:
            self.L.slab_engine_destroy(h)
            self.h = None

    def timings(self):
        """Device milliseconds of the last factor/solve phases (slab_engine_timings)."""
        buf = (ctypes.c_double * 6)()
        self.L.slab_engine_timings(self.h, buf, 6)
        keys = ('leaf_ms', 'tree_ms', 'interface_ms', 'solve_ms', 'apply_ms', 'n_apply')
        return dict(zip(keys, list(buf)))

    @property
    def factor_bytes(self):
        return int(self.L.slab_engine_factor_bytes(self.h))

    @property
    def solve_bytes(self):
        """Bytes of stored factors one solve application reads (slab_engine_solve_bytes)."""
        return int(self.L.slab_engine_solve_bytes(self.h))

    def factor(self, c11=None, c22=None, c1=None, c2=None, c=None, c12=None):
        """Coefficients: device float64 tensors with nleaf*p*p entries (or None);
        c12 (the mixed derivative) only, and always, for an engine made with mixed=True."""
        if (c12 is not None) != self.mixed:
            raise ValueError('c12 goes with SlabEngine(mixed=True), and such an engine needs it')
        args = []
        for t in (c11, c22, c1, c2, c, c12):
            if t is not None:
                t = t.reshape(-1)
                assert t.dtype == torch.float64 and t.is_cuda and t.numel() == self.npts and t.is_contiguous()
            args.append(t)
        self._coef = args  # keep alive until the factorization has read them
        self.generation = getattr(self, 'generation', 0) + 1
        if self.mixed:
            a11, a22, a1, a2, a0, a12 = [_lib.ptr(t) for t in args]
            st = self.L.slab_engine_factor_mixed(self.h, a11, a22, a12, a1, a2, a0)
            return _lib.check(st, 'slab_engine_factor_mixed')
        st = self.L.slab_engine_factor(self.h, *[_lib.ptr(t) for t in args[:5]])
        return _lib.check(st, 'slab_engine_factor')

    def solve(self, bnd, fbody=None, tol=1e-10, max_iter=20, want_faces=False, allow_noconv=False, want_leaf=True):
        """bnd: (ntot,) or (ntot, nrhs) face values (only Dirichlet faces are read).

        Returns (u_leaf (npts, nrhs) device tensor or None if not want_leaf, u_faces
        or None, iters, stats dict).
        """
        dev = bnd.device
        nrhs = 1 if bnd.dim() == 1 else bnd.shape[1]
        if not (want_leaf or want_faces):
            raise ValueError('solve: ask for the leaf-node solution, the face solution or both')
        bnd_cm = _col_major(bnd.to(torch.float64), self.ntot)
        fb_cm = None if fbody is None else _col_major(fbody.to(torch.float64), self.npts)
        uleaf = torch.empty(nrhs, self.npts, dtype=torch.float64, device=dev) if want_leaf else None
        ufaces = torch.empty(nrhs, self.ntot, dtype=torch.float64, device=dev) if want_faces else None
        iters = ctypes.c_int(0)
        stats = (ctypes.c_double * 5)()
        st = self.L.slab_engine_solve(self.h, nrhs, _lib.ptr(bnd_cm), _lib.ptr(fb_cm), float(tol), int(max_iter),
                                      _lib.ptr(ufaces), _lib.ptr(uleaf), ctypes.byref(iters), stats)
        _lib.check(st, 'slab_engine_solve', allow=(_lib.SLAB_ERR_NOCONV,) if allow_noconv else ())
        info = dict(rel_correction=stats[0], residual=stats[1], residual0=stats[2], resloc=stats[3],
                    rel_residual=stats[4], converged=(st == _lib.SLAB_OK))
        return (None if uleaf is None else uleaf.T), (None if ufaces is None else ufaces.T), iters.value, info

    def adjoint(self, gleaf=None, gfaces=None, tol=1e-10, max_iter=20, want_faces=False, want_bnd=True,
                allow_noconv=False):
        """Transposed solve with the stored factors (slab_engine_adjoint).

        gleaf: (npts, nrhs) dL/du at the leaf nodes; gfaces: (ntot, nrhs) dL/du_faces.
        Returns (lam_leaf (npts, nrhs) = dL/dfbody, lam_faces or None,
        gbnd (ntot, nrhs) = dL/dbnd or None, iters, stats dict).
        """
        ref = gleaf if gleaf is not None else gfaces
        nrhs = 1 if ref.dim() == 1 else ref.shape[1]
        dev = ref.device
        gl = None if gleaf is None else _col_major(gleaf.to(torch.float64), self.npts)
        gf = None if gfaces is None else _col_major(gfaces.to(torch.float64), self.ntot)
        lam = torch.empty(nrhs, self.npts, dtype=torch.float64, device=dev)
        lamf = torch.empty(nrhs, self.ntot, dtype=torch.float64, device=dev) if want_faces else None
        gb = torch.empty(nrhs, self.ntot, dtype=torch.float64, device=dev) if want_bnd else None
        iters = ctypes.c_int(0)
        stats = (ctypes.c_double * 5)()
        st = self.L.slab_engine_adjoint(self.h, nrhs, _lib.ptr(gl), _lib.ptr(gf), float(tol), int(max_iter),
                                        _lib.ptr(lam), _lib.ptr(lamf), _lib.ptr(gb), ctypes.byref(iters), stats)
        _lib.check(st, 'slab_engine_adjoint', allow=(_lib.SLAB_ERR_NOCONV,) if allow_noconv else ())
        info = dict(rel_correction=stats[0], residual=stats[1], residual0=stats[2], rel_residual=stats[4],
                    converged=(st == _lib.SLAB_OK))
        t = lambda x: None if x is None else x.T
        return lam.T, t(lamf), t(gb), iters.value, info

    def coeff_grad(self, ufaces, uleaf, lam_leaf, keys=('c',)):
        """dL/d(coefficient) at the leaf nodes for each key in keys (slab_engine_coeff_grad).

        ufaces (ntot, nrhs), uleaf (npts, nrhs): forward solution; lam_leaf
        (npts, nrhs) from adjoint().  Returns {key: (npts,) tensor}, summed over rhs.
        """
        order = ('c11', 'c22', 'c12', 'c1', 'c2', 'c') if self.mixed else ('c11', 'c22', 'c1', 'c2', 'c')
        for k in keys:
            if k not in order:
                raise ValueError(f'unknown coefficient {k}' + (' (c12 needs SlabEngine(mixed=True))'
                                                               if k == 'c12' else ''))
        nrhs = 1 if uleaf.dim() == 1 else uleaf.shape[1]
        uf = _col_major(ufaces.to(torch.float64), self.ntot)
        ul = _col_major(uleaf.to(torch.float64), self.npts)
        lm = _col_major(lam_leaf.to(torch.float64), self.npts)
        out = {k: torch.empty(self.npts, dtype=torch.float64, device=ul.device) for k in keys}
        fn = self.L.slab_engine_coeff_grad_mixed if self.mixed else self.L.slab_engine_coeff_grad
        st = fn(self.h, nrhs, _lib.ptr(uf), _lib.ptr(ul), _lib.ptr(lm), *[_lib.ptr(out.get(k)) for k in order])
        _lib.check(st, 'slab_engine_coeff_grad_mixed' if self.mixed else 'slab_engine_coeff_grad')
        return out

    def residual(self, ufaces, uint, fbody=None):
        """FP64 residual of the full collocation system.

        ufaces: (ntot, nrhs); uint: (nleaf, nrhs, (p-2)^2) leaf-major interior values.
        Returns (r_int like uint, r_faces (ntot, nrhs)).
        """
        nrhs = 1 if ufaces.dim() == 1 else ufaces.shape[1]
        uf = _col_major(ufaces.to(torch.float64), self.ntot)
        ui = uint.to(torch.float64).contiguous()
        fb = None if fbody is None else _col_major(fbody.to(torch.float64), self.npts)
        rint = torch.empty_like(ui)
        rf = torch.empty_like(uf)
        st = self.L.slab_engine_residual(self.h, nrhs, _lib.ptr(uf), _lib.ptr(ui), _lib.ptr(fb), _lib.ptr(rint),
                                         _lib.ptr(rf))
        _lib.check(st, 'slab_engine_residual')
        return rint, rf.T

    def apply(self, rint, rfaces):
        """One application of the factorization (slab_engine_apply): the correction
        M^-1 (rint, rfaces) of one refinement step.  rint: (nleaf, nrhs, (p-2)^2)
        leaf-major like residual(); rfaces: (ntot, nrhs).  Returns (dint like rint,
        dfaces (ntot, nrhs))."""
        nrhs = 1 if rfaces.dim() == 1 else rfaces.shape[1]
        rf = _col_major(rfaces.to(torch.float64), self.ntot)
        ri = rint.to(torch.float64).contiguous()
        if ri.numel() != self.nleaf * nrhs * self.n_int:
            raise ValueError('rint must hold nleaf x nrhs x (p-2)^2 values')
        dint = torch.empty_like(ri)
        df = torch.empty_like(rf)
        st = self.L.slab_engine_apply(self.h, nrhs, _lib.ptr(ri), _lib.ptr(rf), _lib.ptr(dint), _lib.ptr(df))
        _lib.check(st, 'slab_engine_apply')
        return dint, df.T



class SolveGraph:
    """The refined solves of several factored engines as one CUDA graph
    (slab_solve_graph_create / _launch / _status): per engine a conditional
    WHILE node runs the refinement steps, decided on the device, so a launch
    makes no host round trip between steps and the engines' solves run side by
    side.  Inputs and outputs are persistent device buffers owned here:

        g = SolveGraph([e1, e2], nrhs=[1, 4])
        g.set_inputs(0, bnd1); g.set_inputs(1, bnd2)
        g.launch()
        u1, it1, info1 = g.result(0)      # (npts, nrhs) on engine 0's leaf nodes

    The graph reads the engines' current factors (re-factoring with the same
    coefficient set needs no new graph); it must be rebuilt once an engine has
    reallocated its solve buffers (a solve with more right-hand sides)."""

    def __init__(self, engines, nrhs=1, with_fbody=False, tol=1e-10, max_iter=20):
        self.engines = list(engines)
        k = len(self.engines)
        self.nrhs = [int(nrhs)] * k if np.isscalar(nrhs) else [int(r) for r in nrhs]
        if len(self.nrhs) != k:
            raise ValueError('SolveGraph: one nrhs per engine')
        dev = torch.device('cuda', torch.cuda.current_device())
        z = lambda r, m: torch.zeros(r, m, dtype=torch.float64, device=dev)
        self.bnd = [z(r, e.ntot) for e, r in zip(self.engines, self.nrhs)]
        self.fbody = [z(r, e.npts) for e, r in zip(self.engines, self.nrhs)] if with_fbody else None
        self.uleaf = [z(r, e.npts) for e, r in zip(self.engines, self.nrhs)]
        self.L = _lib.lib()
        arr = lambda ts: (ctypes.c_void_p * k)(*[_lib.ptr(t) for t in ts])
        handle = ctypes.c_void_p()
        st = self.L.slab_solve_graph_create(ctypes.byref(handle), (ctypes.c_void_p * k)(*[e.h for e in self.engines]),
                                            k, (ctypes.c_int * k)(*self.nrhs), arr(self.bnd),
                                            None if self.fbody is None else arr(self.fbody), arr(self.uleaf),
                                            float(tol), int(max_iter))
        _lib.check(st, 'slab_solve_graph_create')
        self.h = handle

    def __del__(self):
        h = getattr(self, 'h', None)
        if h is not None and h.value:
            self.L.slab_solve_graph_destroy(h)
            self.h = None

    def set_inputs(self, i, bnd, fbody=None):
        """bnd: (ntot,) or (ntot, nrhs) face values of engine i; fbody: (npts,) or (npts, nrhs)."""
        self.bnd[i].copy_(_col_major(bnd.to(torch.float64), self.engines[i].ntot))
        if fbody is not None:
            if self.fbody is None:
                raise ValueError('SolveGraph made without body loads (with_fbody=False)')
            self.fbody[i].copy_(_col_major(fbody.to(torch.float64), self.engines[i].npts))

    def launch(self, stream=None):
        """Asynchronous on stream (default: torch's current stream)."""
        stream = stream if stream is not None else torch.cuda.current_stream()
        _lib.check(self.L.slab_solve_graph_launch(self.h, ctypes.c_void_p(stream.cuda_stream)),
                   'slab_solve_graph_launch')

    def result(self, i, allow_noconv=False):
        """(u_leaf (npts, nrhs), iters, stats dict) of engine i from the last launch."""
        iters = ctypes.c_int(0)
        stats = (ctypes.c_double * 5)()
        st = self.L.slab_solve_graph_status(self.h, int(i), ctypes.byref(iters), stats)
        _lib.check(st, 'slab_solve_graph_status', allow=(_lib.SLAB_ERR_NOCONV,) if allow_noconv else ())
        info = dict(rel_correction=stats[0], residual=stats[1], residual0=stats[2], resloc=stats[3],
                    rel_residual=stats[4], converged=(st == _lib.SLAB_OK))
        return self.uleaf[i].T, iters.value, info


def leaf_dtn(coeffs, p, D, Dsq, Nx, precision='fp64', return_S=False, interp=None, jxreorder=None):
    """Batched leaf DtN maps (form_DtNs 'build') through slab_leaf_dtn.

    coeffs: dict of device float64 tensors (nleaf, p*p) for 'c11','c22','c1','c2','c'
    and optionally 'c12' (mixed derivative: then interp = HPS_Disc.Interp_mat and
    jxreorder = JJ.Jxreorder are needed, and slab_leaf_dtn_mixed runs).
    Returns DtN (nleaf, 4(p-2), 4(p-2)) float64 on the device (and S if asked).
    """
    L = _lib.lib()
    ref = next(v for v in coeffs.values() if v is not None)
    nleaf = ref.shape[0]
    dev = ref.device
    q = p - 2
    prec = _lib.PREC[precision]
    if coeffs.get('c12') is not None:
        return _leaf_dtn_mixed(L, coeffs, nleaf, p, D, Dsq, Nx, prec, return_S, interp, jxreorder, dev)
    wb = int(L.slab_leaf_dtn_work_bytes(nleaf, p, prec))
    work = torch.empty(wb, dtype=torch.uint8, device=dev)
    dtn = torch.empty(nleaf, 4 * q, 4 * q, dtype=torch.float64, device=dev)
    S = torch.empty(nleaf, q * q, 4 * q, dtype=torch.float64, device=dev) if return_S else None
    info = torch.zeros(nleaf, dtype=torch.int32, device=dev)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    Dd, Dsqd, Nxd = t(D), t(Dsq), t(Nx)
    cs = [coeffs.get(k) for k in ('c11', 'c22', 'c1', 'c2', 'c')]
    cs = [None if c is None else c.to(torch.float64).contiguous() for c in cs]
    st = L.slab_leaf_dtn(nleaf, p, *[_lib.ptr(c) for c in cs], _lib.ptr(Dd), _lib.ptr(Dsqd), _lib.ptr(Nxd), prec,
                         _lib.ptr(work), wb, _lib.ptr(dtn), _lib.ptr(S), _lib.ptr(info),
                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(st, 'slab_leaf_dtn')
    return (dtn, S, info) if return_S else (dtn, info)


def _leaf_dtn_mixed(L, coeffs, nleaf, p, D, Dsq, Nx, prec, return_S, interp, jxreorder, dev):
    if interp is None or jxreorder is None:
        raise ValueError('a mixed derivative (c12) needs interp (Interp_mat) and jxreorder (Jxreorder)')
    q = p - 2
    wb = int(L.slab_leaf_dtn_mixed_work_bytes(nleaf, p, prec))
    work = torch.empty(wb, dtype=torch.uint8, device=dev)
    dtn = torch.empty(nleaf, 4 * q, 4 * q, dtype=torch.float64, device=dev)
    S = torch.empty(nleaf, q * q, 4 * q, dtype=torch.float64, device=dev) if return_S else None
    info = torch.zeros(nleaf, dtype=torch.int32, device=dev)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    Dd, Dsqd, Nxd, Id = t(D), t(Dsq), t(Nx), t(interp)
    jx = torch.as_tensor(np.ascontiguousarray(jxreorder), dtype=torch.int32, device=dev)
    cs = [coeffs.get(k) for k in ('c11', 'c22', 'c12', 'c1', 'c2', 'c')]
    cs = [None if c is None else c.to(torch.float64).contiguous() for c in cs]
    st = L.slab_leaf_dtn_mixed(nleaf, p, *[_lib.ptr(c) for c in cs], _lib.ptr(Dd), _lib.ptr(Dsqd), _lib.ptr(Nxd),
                               _lib.ptr(Id), _lib.ptr(jx), prec, _lib.ptr(work), wb, _lib.ptr(dtn), _lib.ptr(S),
                               _lib.ptr(info), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(st, 'slab_leaf_dtn_mixed')
    return (dtn, S, info) if return_S else (dtn, info)
