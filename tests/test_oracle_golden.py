"""The C oracle against the reference's own outputs (golden fixtures made by
running the unmodified reference) and the MAD-X values its tests pin."""
import numpy as np
import pytest

import helpers as H


@pytest.mark.parametrize('name', [c['name'] for c in H.cases('track')])
def test_oracle_tracks_bit_exact(name):
    c = H.case(name)
    out = H.oracle_case(c)
    ref = H.arr(name, 'out/tracks')
    assert out['tracks'].shape == ref.shape
    assert np.array_equal(out['tracks'], ref, equal_nan=True)


@pytest.mark.parametrize('name', [c['name'] for c in H.cases('sa')])
def test_oracle_loss_turns_bit_exact(name):
    c = H.case(name)
    out = H.oracle_case(c)
    assert np.array_equal(out['lost'], H.arr(name, 'out/lost'))


def test_oracle_fodo_matches_madx():
    # the reference's tests/tracking.py pin: |dx| < 1e-6 against MAD-X
    meta, _ = H.golden()
    out = H.oracle_case(H.case('fodo_fived'))
    x = np.array(meta['madx']['tracking_fodo_x'])
    assert np.max(np.abs(out['tracks'][0, :, 0] - x)) < 1e-6


def test_golden_has_uneven_survival():
    lost = H.arr('c3_da_sa', 'out/lost')
    assert 0 < np.sum(lost < 512) < lost.size
    assert len(np.unique(lost)) > 10
