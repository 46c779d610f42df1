"""Autotuner for the engine's launch choices.

Each tunable (slab_engine_set_option in include/slablu_gb300.h) is timed on the
engine's own factorization or solve with its candidates, the fastest is kept,
and the choice is cached per (GPU, p, leaf grid, slab width, precision) in a
JSON file (SLAB_TUNE_CACHE, default ~/.cache/slablu_gb300/tune.json), so later
engines on the same shape apply it without timing.

    from slablu_gb300 import autotune
    picks = autotune.tune(engine, dict(c11=one, c22=one, c=c), bnd)
"""
import json
import os

import torch

from . import _lib

# name -> (option key, candidates in order of preference on ties)
TUNABLES = {
    'leaf_ctas': (_lib.SLAB_OPT_LEAF_CTAS, (0, 2, 1)),
    'iface_solve': (_lib.SLAB_OPT_IFACE_SOLVE, (0, 1)),
    'iface_lookahead': (_lib.SLAB_OPT_IFACE_LOOKAHEAD, (1, 0)),
    'tree_tc': (_lib.SLAB_OPT_TREE_TC, (0, 1)),
    'leaf_assembly': (_lib.SLAB_OPT_LEAF_ASSEMBLY, (1, 0)),
    'iface_outer_inv': (_lib.SLAB_OPT_IFACE_OUTER_INV, (1, 0)),
    'iface_panel': (_lib.SLAB_OPT_IFACE_PANEL, (0, 1)),
    'gemm_tiles': (_lib.SLAB_OPT_GEMM_TILES, (0, 1)),
}


def cache_path():
    return os.environ.get('SLAB_TUNE_CACHE',
                          os.path.join(os.path.expanduser('~'), '.cache', 'slablu_gb300', 'tune.json'))


def shape_key(engine):
    g = engine.geom
    dev = torch.cuda.get_device_name() if torch.cuda.is_available() else 'cpu'
    return f'{dev}|p={g.p}|{g.n0}x{g.n1}|buf={g.buf}|{engine.precision}'


def load_cache(path=None):
    path = path or cache_path()
    try:
        with open(path) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def save_cache(data, path=None):
    path = path or cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + '.tmp'
        with open(tmp, 'w') as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home leaves the choices untuned next time, nothing else


def set_options(engine, picks):
    for name, value in picks.items():
        if name in TUNABLES:
            _lib.check(engine.L.slab_engine_set_option(engine.h, TUNABLES[name][0], int(value)),
                       'slab_engine_set_option')


def apply_cached(engine, path=None):
    """Apply the cached choices for this engine's shape; returns them (or None)."""
    picks = load_cache(path).get(shape_key(engine))
    if picks:
        set_options(engine, picks)
    return picks


def _time_leaf(engine, coeffs, reps):
    best = float('inf')
    for _ in range(reps):
        engine.factor(**coeffs)
        best = min(best, engine.timings()['leaf_ms'])
    return best


def _time_interface(engine, coeffs, reps):
    best = float('inf')
    for _ in range(reps):
        engine.factor(**coeffs)
        best = min(best, engine.timings()['interface_ms'])
    return best


def _time_tree_and_interface(engine, coeffs, reps):
    best = float('inf')
    for _ in range(reps):
        engine.factor(**coeffs)
        t = engine.timings()
        best = min(best, t['tree_ms'] + t['interface_ms'])
    return best


def _time_apply(engine, bnd, reps):
    best = float('inf')
    for _ in range(reps):
        engine.solve(bnd, tol=0.0, max_iter=2, allow_noconv=True)
        t = engine.timings()
        if t['n_apply'] > 0:
            best = min(best, t['apply_ms'] / t['n_apply'])
    return best


def _time_tree_and_solve(engine, coeffs, bnd, reps, tol):
    """Merge-tree time plus the refined solve's time: a choice that changes the
    factors' accuracy changes the number of refinement applications too."""
    best = float('inf')
    for _ in range(reps):
        engine.factor(**coeffs)
        t_tree = engine.timings()['tree_ms']
        engine.solve(bnd, tol=tol, max_iter=30, allow_noconv=True)
        best = min(best, t_tree + engine.timings()['solve_ms'])
    return best


def tune(engine, coeffs, bnd, reps=2, use_cache=True, path=None, tol=1e-6):
    """Time the candidates of every tunable on this engine and keep the fastest.

    coeffs: the engine.factor keyword arguments; bnd: a face vector for solve.
    Returns {name: value, ..., 'timings_ms': {...}}; the engine is left
    factored with the chosen options."""
    if use_cache:
        cached = apply_cached(engine, path)
        if cached:
            engine.factor(**coeffs)
            return dict(cached, cached=True)
    picks, timings = {}, {}
    key, cands = TUNABLES['leaf_ctas']
    t_leaf = {}
    for v in cands:
        _lib.check(engine.L.slab_engine_set_option(engine.h, key, v), 'slab_engine_set_option')
        t_leaf[v] = _time_leaf(engine, coeffs, reps)
    picks['leaf_ctas'] = min(cands, key=lambda v: (t_leaf[v], cands.index(v)))
    timings['leaf_ms'] = {str(v): t for v, t in t_leaf.items()}
    _lib.check(engine.L.slab_engine_set_option(engine.h, key, picks['leaf_ctas']), 'slab_engine_set_option')
    if not getattr(engine, 'mixed', False):
        key, cands = TUNABLES['leaf_assembly']
        t_asm = {}
        for v in cands:
            _lib.check(engine.L.slab_engine_set_option(engine.h, key, v), 'slab_engine_set_option')
            t_asm[v] = _time_leaf(engine, coeffs, reps)
        picks['leaf_assembly'] = min(cands, key=lambda v: (t_asm[v], cands.index(v)))
        timings['leaf_assembly_ms'] = {str(v): t for v, t in t_asm.items()}
        _lib.check(engine.L.slab_engine_set_option(engine.h, key, picks['leaf_assembly']), 'slab_engine_set_option')
    if engine.geom.Npan > 2 and engine.precision == 'mixed':
        key, cands = TUNABLES['iface_outer_inv']
        t_oi = {}
        for v in cands:
            _lib.check(engine.L.slab_engine_set_option(engine.h, key, v), 'slab_engine_set_option')
            t_oi[v] = _time_interface(engine, coeffs, reps)
        picks['iface_outer_inv'] = min(cands, key=lambda v: (t_oi[v], cands.index(v)))
        timings['iface_outer_inv_ms'] = {str(v): t for v, t in t_oi.items()}
        _lib.check(engine.L.slab_engine_set_option(engine.h, key, picks['iface_outer_inv']), 'slab_engine_set_option')
    if engine.geom.Npan > 1 and engine.precision in ('mixed', 'fp32'):
        key, cands = TUNABLES['iface_lookahead']
        t_if = {}
        for v in cands:
            _lib.check(engine.L.slab_engine_set_option(engine.h, key, v), 'slab_engine_set_option')
            t_if[v] = _time_interface(engine, coeffs, reps)
        picks['iface_lookahead'] = min(cands, key=lambda v: (t_if[v], cands.index(v)))
        timings['interface_ms'] = {str(v): t for v, t in t_if.items()}
        _lib.check(engine.L.slab_engine_set_option(engine.h, key, picks['iface_lookahead']), 'slab_engine_set_option')
    if engine.geom.Npan > 1 and engine.precision == 'fp32':
        key, cands = TUNABLES['iface_panel']
        t_pn = {}
        for v in cands:
            _lib.check(engine.L.slab_engine_set_option(engine.h, key, v), 'slab_engine_set_option')
            t_pn[v] = _time_interface(engine, coeffs, reps)
        picks['iface_panel'] = min(cands, key=lambda v: (t_pn[v], cands.index(v)))
        timings['iface_panel_ms'] = {str(v): t for v, t in t_pn.items()}
        _lib.check(engine.L.slab_engine_set_option(engine.h, key, picks['iface_panel']), 'slab_engine_set_option')
    if engine.precision != 'fp64':
        key, cands = TUNABLES['gemm_tiles']
        t_gt = {}
        for v in cands:
            _lib.check(engine.L.slab_engine_set_option(engine.h, key, v), 'slab_engine_set_option')
            t_gt[v] = _time_tree_and_interface(engine, coeffs, reps)
        picks['gemm_tiles'] = min(cands, key=lambda v: (t_gt[v], cands.index(v)))
        timings['gemm_tiles_ms'] = {str(v): t for v, t in t_gt.items()}
        _lib.check(engine.L.slab_engine_set_option(engine.h, key, picks['gemm_tiles']), 'slab_engine_set_option')
    if engine.precision != 'fp64':
        key, cands = TUNABLES['tree_tc']
        t_tc = {}
        for v in cands:
            _lib.check(engine.L.slab_engine_set_option(engine.h, key, v), 'slab_engine_set_option')
            t_tc[v] = _time_tree_and_solve(engine, coeffs, bnd, reps, tol)
        picks['tree_tc'] = min(cands, key=lambda v: (t_tc[v], cands.index(v)))
        timings['tree_plus_solve_ms'] = {str(v): t for v, t in t_tc.items()}
        _lib.check(engine.L.slab_engine_set_option(engine.h, key, picks['tree_tc']), 'slab_engine_set_option')
    engine.factor(**coeffs)
    key, cands = TUNABLES['iface_solve']
    if engine.geom.Npan > 1:
        t_app = {}
        for v in cands:
            _lib.check(engine.L.slab_engine_set_option(engine.h, key, v), 'slab_engine_set_option')
            t_app[v] = _time_apply(engine, bnd, reps)
        picks['iface_solve'] = min(cands, key=lambda v: (t_app[v], cands.index(v)))
        timings['apply_ms'] = {str(v): t for v, t in t_app.items()}
        _lib.check(engine.L.slab_engine_set_option(engine.h, key, picks['iface_solve']), 'slab_engine_set_option')
    if use_cache:
        data = load_cache(path)
        data[shape_key(engine)] = dict(picks)
        save_cache(data, path)
    return dict(picks, timings_ms=timings, cached=False)
