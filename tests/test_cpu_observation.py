"""Result packing (a16): the sample container the pool returns -- the
reference's ObservationList when qgate is importable, else the package's own
with the same constructor and accessors (qgate/simulator/observation.py:53-100)."""
import numpy as np
import pytest

from qgate_gb300 import observation


def test_observation_list_accessors():
    if observation.ObservationList.__module__ != 'qgate_gb300.observation':
        pytest.skip('the reference ObservationList is in use')
    refs = ['a', 'b', 'c']
    vals = np.array([0b001, 0b011, 0b000, 0b001], np.int64)
    obs = observation.ObservationList(refs, vals, 0b100)  # 'c' never used
    assert len(obs) == 4 and np.array_equal(obs.intarray, vals)
    item = obs[1]
    assert isinstance(item, observation.Observation) and int(item) == 3 and item.int == 3
    assert (item('a'), item('b'), item('c')) == (1, 1, None)
    assert item == observation.Observation(refs, 3, 0b100)
    with pytest.raises(ValueError, match='int'):
        item == 3  # noqa: B015 (the reference refuses integer comparison)
    sl = obs[1:3]
    assert isinstance(sl, observation.ObservationList) and len(sl) == 2
    assert [int(o) for o in obs] == [1, 3, 0, 1]
    assert obs('a') == [1, 1, 0, 1] and obs('b') == [0, 1, 0, 0]
    assert obs('c') == [None] * 4
    with pytest.raises(RuntimeError, match='unknown ref'):
        obs('d')
    h = obs.histgram()
    assert isinstance(h, observation.ObservationHistgram)
    assert (h[1], h[3], h[0], h[7], h.n_samples, len(h)) == (2, 1, 1, 0, 4, 3)
    assert dict(h.items()) == {1: 2, 3: 1, 0: 1}
