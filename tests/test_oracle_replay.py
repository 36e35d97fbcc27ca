"""Pins the oracle to the reference: the numpy oracle runtime replays every
boundary trace recorded from the reference's own CPU runtime (complex128) and
must reproduce all of its results."""
import numpy as np
import pytest

from oracle import runtime as oracle_rt
from tests import replay


@pytest.mark.parametrize('name', replay.trace_names())
def test_oracle_replays_reference_trace(name):
    calls, arrays = replay.load_trace(name)
    stats = replay.replay(calls, arrays, oracle_rt, np.float64)
    assert not stats.failures, stats.failures[:5]
    assert stats.checks > 0
    # complex128 oracle vs complex128 reference: same formulas, only the
    # summation order differs, so no sampled index may move.
    assert stats.sample_mismatch == 0
