"""Autotuner cache (CPU): keys, JSON round trip, unknown names ignored."""
import types

from slablu_gb300 import autotune


def _fake_engine():
    g = types.SimpleNamespace(p=22, n0=100, n1=100, buf=10, Npan=10)
    calls = []
    lib = types.SimpleNamespace(slab_engine_set_option=lambda h, k, v: calls.append((k, v)) or 0)
    return types.SimpleNamespace(geom=g, precision='mixed', L=lib, h=None), calls


def test_cache_round_trip(tmp_path):
    path = str(tmp_path / 'tune.json')
    eng, calls = _fake_engine()
    assert autotune.apply_cached(eng, path) is None
    data = autotune.load_cache(path)
    data[autotune.shape_key(eng)] = {'leaf_ctas': 2, 'iface_solve': 1, 'unknown': 5}
    autotune.save_cache(data, path)
    picks = autotune.apply_cached(eng, path)
    assert picks['leaf_ctas'] == 2
    assert sorted(calls) == [(autotune.TUNABLES['leaf_ctas'][0], 2), (autotune.TUNABLES['iface_solve'][0], 1)]


def test_shape_key_distinguishes_precision():
    eng, _ = _fake_engine()
    k1 = autotune.shape_key(eng)
    eng.precision = 'fp64'
    assert autotune.shape_key(eng) != k1
    assert 'p=22' in k1 and '100x100' in k1 and 'buf=10' in k1
