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
    assert obs[1] == 3 and len(obs[1:3]) == 2
    assert obs('a') == [1, 1, 0, 1] and obs('b') == [0, 1, 0, 0]
    assert obs('c') == [None] * 4
    with pytest.raises(RuntimeError, match='unknown ref'):
        obs('d')
    assert obs.histgram() == {1: 2, 3: 1, 0: 1}
