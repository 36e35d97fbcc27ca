"""Drop-in parity: every boundary trace recorded from the reference front-end
on the reference's complex128 CPU runtime is replayed against the GB300
runtime, in complex128 (tolerance 1e-11 abs / 1e-9 rel) and complex64
(3e-6 abs / 1e-4 rel), with gate fusion on (default tile) and off.  Sampled
indices must equal the reference's except for uniforms within tau of a CDF
boundary, tau = max |cdf_engine - cdf_reference|."""
import numpy as np
import pytest

from tests import replay

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('fusion', [0, 1], ids=['fused', 'unfused'])
@pytest.mark.parametrize('dtype', [np.float64, np.float32], ids=['c128', 'c64'])
@pytest.mark.parametrize('name', replay.trace_names())
def test_replay_reference_trace(rt, name, dtype, fusion):
    from qgate_gb300 import _native as nat
    nat.set_fusion(fusion)
    try:
        calls, arrays = replay.load_trace(name)
        stats = replay.replay(calls, arrays, rt, dtype)
    finally:
        nat.set_fusion(0)
    assert not stats.failures, stats.failures[:5]
    assert stats.sample_mismatch_outside_tol == 0


@pytest.mark.parametrize('dtype', [np.float64, np.float32], ids=['c128', 'c64'])
def test_replay_reference_traces_through_trace_replay(rt, dtype):
    """Every trace replayed three times in a row with trace replay on (the
    default): runs of gates that recur between observations are captured
    into CUDA graphs the second time and replayed the third, and every
    result still matches the reference's."""
    from qgate_gb300 import _native as nat
    nat.set_fusion(0)
    nat.set_trace_replay(True)
    nat.trace_stats(reset=True)
    for name in replay.trace_names():
        calls, arrays = replay.load_trace(name)
        for _ in range(3):
            stats = replay.replay(calls, arrays, rt, dtype)
            assert not stats.failures, (name, stats.failures[:5])
            assert stats.sample_mismatch_outside_tol == 0, name
    st = nat.trace_stats(reset=True)
    assert st['captures'] > 0 and st['hits'] > 0, st
