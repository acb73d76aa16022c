"""Batched error seeds: one persistent launch (CUDA graph, LPT order, tuned
grid) over many lattice seeds with uneven particle and turn counts must give
exactly the results of one launch per seed and of the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(flags_extra=0, n_seeds=12, seed=3):
    import ufo_gb300 as u
    from ufo_gb300 import workloads as W
    ring = W.c1_ring(u)
    params = W.c4_parameters(ring)
    rows = W.c4_seed_rows(ring, n_seeds, seed=seed)
    rng = np.random.default_rng(seed)
    parts = rng.integers(20, 200, n_seeds)
    turns = rng.integers(30, 120, n_seeds)
    b = u.TrackBatch(ring, params, rows, parts, turns, flags=u.KICK | flags_extra)
    b.coords[:] = W.c1_beam(b.n, seed=seed) * 25
    return ring, params, rows, b


def test_batched_graph_equals_one_launch_per_seed():
    _, _, _, b = _batch()
    f_plain, l_plain = [a.copy() for a in b.run_plain()]
    f_batch, l_batch = b.run(graph=True)
    assert np.array_equal(l_batch, l_plain)
    assert np.array_equal(f_batch, f_plain, equal_nan=True)
    # the graph replays on the same buffers
    b.launch(graph=True)
    f2, l2 = b.download()
    assert np.array_equal(f2, f_batch, equal_nan=True)


def test_batched_vs_oracle_subset():
    import ufo_gb300 as u
    from oracle import oracle as O
    ring, params, rows, b = _batch(n_seeds=6, seed=5)
    final, lost = b.run()
    idx = np.random.default_rng(0).choice(b.n, 48, replace=False)
    for i in idx:
        ref = O.track(ring, u.KICK, b.coords[i:i + 1], int(b.pturns[i]), parameters=params,
                      where=[-1], seed=[int(b.seed[i])], seed_values=rows, tracks=False)
        assert np.array_equal(final[i], ref['final'][0], equal_nan=True)
        assert lost[i] == ref['lost'][0]


def test_autotune_keeps_results(tmp_path, monkeypatch):
    import ufo_gb300 as u
    monkeypatch.setenv('UFO_GB300_CACHE', str(tmp_path))
    _, _, _, b = _batch(flags_extra=u.FMA, n_seeds=8, seed=7)
    ref_f, ref_l = [a.copy() for a in b.run_plain()]
    best = u.autotune(b, warps=(8, 16), scale=8)
    assert best['warps_per_sm'] in (8, 16) and best['order'] in ('lpt', 'seed')
    f, l = b.run()
    assert np.array_equal(l, ref_l)
    assert np.array_equal(f, ref_f, equal_nan=True)
    again = u.autotune(b, warps=(8, 16), scale=8)  # served from the cache
    assert again['warps_per_sm'] == best['warps_per_sm']
    from ufo_gb300 import capi
    capi.check(capi.load().ufo_ctx_set_tuning(b.ctx.handle, 16))
