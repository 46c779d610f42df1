"""ctypes binding of the C ABI in include/slablu_gb300.h.

The shared library is built in-tree (``python -m slablu_gb300.build``).  There
is no CPU fallback: if the library is missing every entry point raises.
"""
import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libslablu_gb300.so')
HEADER = os.path.join(os.path.dirname(HERE), 'include', 'slablu_gb300.h')

SLAB_OK = 0
SLAB_ERR_NOCONV = -5
PREC = {'fp64': 0, 'mixed': 1, 'fp32': 2}

_lib = None

c_int, c_ll, c_double, c_size, c_void = ctypes.c_int, ctypes.c_longlong, ctypes.c_double, ctypes.c_size_t, ctypes.c_void_p
P_int = ctypes.POINTER(ctypes.c_int)
P_double = ctypes.POINTER(ctypes.c_double)

_SIGS = {
    'slab_version': (c_int, []),
    'slab_last_error': (ctypes.c_char_p, []),
    'slab_leaf_dtn_work_bytes': (c_size, [c_int, c_int, c_int]),
    'slab_leaf_dtn': (c_int, [c_int, c_int] + [c_void] * 8 + [c_int, c_void, c_size, c_void, c_void, c_void, c_void]),
    'slab_engine_create': (c_int, [ctypes.POINTER(c_void), c_int, c_int, c_int, c_int, c_int,
                                   P_double, P_double, P_double, P_double, P_int, c_void]),
    'slab_engine_create_mixed': (c_int, [ctypes.POINTER(c_void), c_int, c_int, c_int, c_int, c_int,
                                         P_double, P_double, P_double, P_double, P_int, c_void]),
    'slab_engine_destroy': (c_int, [c_void]),
    'slab_engine_nfaces': (c_ll, [c_void]),
    'slab_engine_nleaves': (c_ll, [c_void]),
    'slab_engine_factor': (c_int, [c_void] * 6),
    'slab_engine_factor_mixed': (c_int, [c_void] * 7),
    'slab_engine_solve': (c_int, [c_void, c_int, c_void, c_void, c_double, c_int, c_void, c_void, P_int, P_double]),
    'slab_engine_residual': (c_int, [c_void, c_int] + [c_void] * 5),
    'slab_engine_apply': (c_int, [c_void, c_int] + [c_void] * 4),
    'slab_solve_graph_create': (c_int, [ctypes.POINTER(c_void), c_void, c_int, c_void, c_void, c_void, c_void,
                                        c_double, c_int]),
    'slab_solve_graph_launch': (c_int, [c_void, c_void]),
    'slab_solve_graph_status': (c_int, [c_void, c_int, P_int, P_double]),
    'slab_solve_graph_destroy': (c_int, [c_void]),
    'slab_engine_adjoint': (c_int, [c_void, c_int, c_void, c_void, c_double, c_int, c_void, c_void, c_void,
                                    P_int, P_double]),
    'slab_engine_coeff_grad': (c_int, [c_void, c_int] + [c_void] * 8),
    'slab_engine_coeff_grad_mixed': (c_int, [c_void, c_int] + [c_void] * 9),
    'slab_engine_factor_bytes': (c_size, [c_void]),
    'slab_engine_solve_bytes': (c_size, [c_void]),
    'slab_engine_timings': (c_int, [c_void, P_double, c_int]),
    'slab_leaf_dtn_noalloc_max_bytes': (c_size, []),
    'slab_leaf_dtn_noalloc': (c_int, [c_int, c_int] + [c_void] * 8 + [c_int, c_void, c_void, c_void]),
    'slab_launch_count': (c_ll, []),
    'slab_dgemm_emu_work_bytes': (c_size, [c_int, c_int, c_int]),
    'slab_engine_set_option': (c_int, [c_void, c_int, c_int]),
    'slab_engine_get_option': (c_int, [c_void, c_int]),
    'slab_dgemm_emu': (c_int, [c_int, c_int, c_int, c_double, c_void, c_int, c_void, c_int, c_double, c_void, c_int,
                               c_void, c_size, c_void]),
    'slab_csr_assemble': (c_int, [c_ll, c_void, c_void, c_ll, c_void, c_void]),
    'slab_leaf_dtn_mixed_work_bytes': (c_size, [c_int, c_int, c_int]),
    'slab_leaf_dtn_mixed': (c_int, [c_int, c_int] + [c_void] * 11 + [c_int, c_void, c_size, c_void, c_void, c_void,
                                                                      c_void]),
    'slab_csr_spmv': (c_int, [c_int, c_void, c_void, c_void, c_void, c_double, c_double, c_void, c_void]),
    'slab_dense_lu_work_bytes': (c_size, [c_int]),
    'slab_dense_lu': (c_int, [c_int, c_void, c_int, c_void, c_size, P_int, c_void]),
    'slab_dense_lu_solve': (c_int, [c_int, c_int, c_void, c_int, c_void, c_void, c_int, c_void, c_int, c_void]),
    'slab_sgemm_tc_work_bytes': (c_size, [c_int, c_int, c_int, c_int]),
    'slab_sgemm_tc': (c_int, [c_int, c_int, c_int, ctypes.c_float, c_void, c_int, c_ll, c_void, c_int, c_ll,
                              ctypes.c_float, c_void, c_int, c_ll, c_int, c_void, c_size, c_void]),
}


SLAB_OPT_LEAF_CTAS = 1
SLAB_OPT_IFACE_SOLVE = 2
SLAB_OPT_IFACE_LOOKAHEAD = 3
SLAB_OPT_TREE_TC = 4
SLAB_OPT_LEAF_ASSEMBLY = 5
SLAB_OPT_IFACE_OUTER_INV = 6
SLAB_OPT_IFACE_PANEL = 7
SLAB_OPT_GEMM_TILES = 8


class SlabError(RuntimeError):
    def __init__(self, what, status):
        msg = lib().slab_last_error().decode(errors='replace')
        super().__init__(f'{what} failed with status {status}: {msg}')
        self.status = status


def header_symbols():
    """Function names declared in include/slablu_gb300.h."""
    with open(HEADER) as f:
        text = f.read()
    return sorted(set(re.findall(r'\b(slab_[a-z0-9_]+)\s*\(', text)))


def lib():
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f'{LIB_PATH} is missing: build it with `python -m slablu_gb300.build` '
                              '(slablu_gb300 has no CPU fallback)')
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status, what, allow=()):
    if status != SLAB_OK and status not in allow:
        raise SlabError(what, status)
    return status


def ptr(t):
    """Device (or host) address of a tensor, or None."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def np_ptr(a, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))
