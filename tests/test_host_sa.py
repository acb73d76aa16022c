"""StableAperture.run's host logic without a GPU: which launches each
compaction mode makes and how the two-phase run stitches its phases together.

The launches are replaced by a stand-in for capi.track that loses particle i
at turn lost_at[i] (its first `turns` turns counted from the start of that
launch) and records every call, so the tests check the turn numbers, flags and
tuning each mode passes to the library and the loss turns and coordinates it
returns (ufo/sa.py:18-145 defines the quantities)."""
import numpy as np
import pytest


class FakeContext:
    device = 0
    warps_per_sm = 16

    def __init__(self):
        self.tunings = []

    def set_tuning(self, w):
        self.tunings.append(int(w))
        self.warps_per_sm = int(w)


@pytest.fixture
def fake_library(monkeypatch):
    from ufo_gb300 import capi, drivers
    calls = []
    state = {}

    def track(ctx, dprog, coords, turns, mode=0, flags=0, seed=None, pturns=None, slots=0,
              every=1, want_tracks=True, want_final=True):
        coords = np.asarray(coords)
        # a particle's identity travels in its x coordinate (phase 2 gets the
        # survivors' final coordinates, which keep it)
        ids = coords[:, 0].astype(np.int64)
        left = state['lost_at'][ids] - state['offset'].get(len(calls), 0)
        lost = np.where(left < turns, left, turns).astype(np.uint32)
        final = coords.copy()
        final[:, 1] = final[:, 1] + lost       # something that depends on the turns run
        calls.append({'turns': turns, 'mode': mode, 'flags': flags, 'n': len(coords),
                      'tuning': ctx.warps_per_sm})
        return None, lost, final

    monkeypatch.setattr(capi, 'track', track)
    monkeypatch.setattr(drivers._Compiled, 'device', lambda self, ctx, seed_values: object())
    monkeypatch.setattr(drivers, '_sm_count', lambda device: 152)
    return calls, state


def _sa(line, n, T):
    import ufo_gb300 as u
    sa = u.StableAperture(line, flags=u.KICK | u.DOUBLE_PRECISION, turns=T, particles=n,
                          parameters=['x', 'px'], context=FakeContext())
    sa.parameters[:, 0] = np.arange(n)
    sa.parameters[:, 1] = 0.0
    return sa


def _ring():
    import ufo_gb300 as u
    return u.Line('cell', [u.Drift('d', length=1.0),
                           u.Quadrupole('q', length=0.2, k1=0.5),
                           u.Drift('d2', length=1.0)])


def test_default_is_two_phase_and_stitches_turns(fake_library):
    from ufo_gb300 import capi
    calls, state = fake_library
    n, T = 6000, 800
    rng = np.random.default_rng(3)
    lost_at = np.where(rng.random(n) < 0.3, T, rng.integers(0, T, n))
    state['lost_at'] = lost_at
    state['offset'] = {1: T // 8}             # phase 2 starts T/8 turns later
    sa = _sa(_ring(), n, T)
    sa.run()
    assert [c['turns'] for c in calls] == [T // 8, T - T // 8]
    assert all(c['mode'] == capi.UFO_MODE_SA for c in calls)
    assert not any(c['flags'] & capi.UFO_TRACK_COMPACT for c in calls)
    alive = lost_at >= T // 8
    assert calls[1]['n'] == int(alive.sum())
    # the survivors' grid: about 0.9 of its warps per SM, at least 2
    expect = int(min(16, max(2, round(alive.sum() / (0.9 * 32 * 152)))))
    assert calls[1]['tuning'] == expect
    assert sa.ctx.warps_per_sm == 16          # tuning restored
    assert np.array_equal(sa.lost, np.minimum(lost_at, T))
    assert np.array_equal(sa.final[:, 1], np.minimum(lost_at, T))


def test_compact_true_is_one_compacting_launch(fake_library):
    import ufo_gb300 as u
    from ufo_gb300 import capi
    calls, state = fake_library
    n, T = 500, 300
    state['lost_at'] = np.arange(n) % (T + 50)
    state['offset'] = {}
    sa = _sa(_ring(), n, T)
    sa.run(compact=True)
    assert len(calls) == 1
    assert calls[0]['turns'] == T
    assert calls[0]['flags'] & capi.UFO_TRACK_COMPACT
    assert calls[0]['tuning'] == u.StableAperture.COMPACT_WARPS_PER_SM
    assert sa.ctx.warps_per_sm == 16
    assert np.array_equal(sa.lost, np.minimum(state['lost_at'], T))


def test_turn_reading_lattice_never_splits(fake_library):
    """A lattice that reads `turn` (here a time-dependent kicker) would see
    its turn numbers restart in a second launch: the default and an explicit
    two-phase request both make one compacting launch."""
    import ufo_gb300 as u
    import kickers
    from ufo_gb300 import capi
    calls, state = fake_library
    n, T = 400, 200
    state['lost_at'] = np.arange(n) % (T + 10)
    state['offset'] = {}
    kick = kickers.NLKGate('nlk', knl=[0.0, 0.5, 0.0], ksl=[0.0])
    line = u.Line('ring', [kick] + list(_ring().flatten()))
    for compact in (None, 'two-phase'):
        calls.clear()
        sa = _sa(line, n, T)
        assert sa._uses_turn()
        sa.run(compact=compact)
        assert len(calls) == 1 and calls[0]['turns'] == T
        assert calls[0]['flags'] & capi.UFO_TRACK_COMPACT


def test_compact_false_is_one_plain_persistent_launch(fake_library):
    from ufo_gb300 import capi
    calls, state = fake_library
    n, T = 300, 100
    state['lost_at'] = np.arange(n)
    state['offset'] = {}
    sa = _sa(_ring(), n, T)
    sa.run(compact=False)
    assert len(calls) == 1 and calls[0]['turns'] == T
    assert not calls[0]['flags'] & capi.UFO_TRACK_COMPACT
    assert calls[0]['tuning'] == 16
