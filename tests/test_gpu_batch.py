"""GPU parity of batched uneven circuits (sum_i <Z_i> per circuit) against
the oracle's complex128 runs."""
import numpy as np
import pytest

from oracle import statevec as sv

pytestmark = pytest.mark.gpu


def _oracle_sum_z(n, ops):
    psi = sv.run_ops(n, [('g', nm, a, False, t, c) for nm, a, t, c in ops], np.complex128)
    return sum(2 * sv.calc_probability(psi, q) - 1 for q in range(n))


def test_batch_sizes_8_to_20():
    from qgate_gb300.batch import hea_batch, sum_z
    circuits = hea_batch(count=60, seed=3, min_qubits=8, max_qubits=20, min_depth=2, max_depth=6)
    got = sum_z(circuits)
    for (n, ops), g in zip(circuits, got):
        want = _oracle_sum_z(n, ops)
        assert abs(g - want) < 2e-5 * n, (n, g, want)


def test_batch_mixed_gates_and_controls():
    """Dense random gates with controls, every size from 8 to 16."""
    from qgate_gb300.batch import sum_z
    from tests.gpu_helpers import random_ops
    rng = np.random.default_rng(8)
    circuits = []
    for n in range(8, 17):
        ops = [(nm, a, t, c) for _, nm, a, adj, t, c in random_ops(rng, n, 80, max_controls=3)
               if not adj]
        circuits.append((n, ops))
    got = sum_z(circuits)
    for (n, ops), g in zip(circuits, got):
        assert abs(g - _oracle_sum_z(n, ops)) < 2e-5 * n


@pytest.mark.parametrize('one_launch', [1, 0], ids=['one_launch', 'per_round'])
def test_batch_support_growing_over_many_stages(one_launch):
    """Circuits whose nonzero amplitudes spread over the lanes a few at a
    time (gates on the low lanes first, then entangling gates that reach one
    more high lane per stage), so that the stages skip different sets of
    tiles that can still only hold zeros; against the oracle."""
    from qgate_gb300 import _native as nat
    from qgate_gb300.batch import sum_z
    rng = np.random.default_rng(31)
    circuits = []
    for n in (14, 17, 19):
        ops = [('H', (), q, ()) for q in range(12)]
        for hi in range(12, n):
            lo = int(rng.integers(0, 12))
            ops.append(('RY', (float(rng.uniform(0, 3)),), lo, ()))
            ops.append(('X', (), hi, (lo,)))
            ops.append(('RZ', (float(rng.uniform(0, 3)),), hi, ()))
            # a wide gate on low lanes between, so that the next high lane
            # lands in a later stage
            ops += [('X', (), q + 1, (q,)) for q in range(11)]
        circuits.append((n, ops))
    nat.call('qg_set_batch_one_launch', one_launch)
    try:
        got = sum_z(circuits)
    finally:
        nat.call('qg_set_batch_one_launch', 1)
    for (n, ops), g in zip(circuits, got):
        want = _oracle_sum_z(n, ops)
        assert abs(g - want) < 2e-5 * n, (n, g, want)


def test_batch_repeatable_and_order_independent():
    from qgate_gb300.batch import hea_batch, sum_z
    circuits = hea_batch(count=40, seed=4, max_qubits=16)
    a = sum_z(circuits)
    b = sum_z(circuits[::-1])[::-1]
    assert np.array_equal(a, b)


@pytest.mark.parametrize('one_launch', [1, 0], ids=['one_launch', 'per_round'])
def test_batch_circuits_without_gates(one_launch):
    """Circuits with no gates, resident (10 qubits) and staged (15 qubits),
    beside ones with gates: sum_i <Z_i> of |0...0> is n."""
    from qgate_gb300 import _native as nat
    from qgate_gb300.batch import hea_batch, sum_z
    circuits = [(10, []), (15, [])] + hea_batch(count=6, seed=8, min_qubits=13, max_qubits=16)
    nat.call('qg_set_batch_one_launch', one_launch)
    try:
        got = sum_z(circuits)
    finally:
        nat.call('qg_set_batch_one_launch', 1)
    assert got[0] == 10.0 and got[1] == 15.0, got[:2]
    for (n, ops), a in zip(circuits[2:], got[2:]):
        want = _oracle_sum_z(n, ops)
        assert abs(a - want) < 2e-5 * n, (n, a, want)


def test_batch_one_launch_equals_per_round_launches():
    """The batch as one persistent launch over the work queue (default) and as
    one launch per round give the same sums (both against the oracle), for the
    benchmark's mix of 8..20-qubit circuits; the one-launch path ran (a
    single timed launch per call)."""
    from qgate_gb300 import _native as nat
    from qgate_gb300.batch import hea_batch, sum_z
    circuits = hea_batch(count=48, seed=5, min_qubits=8, max_qubits=20, min_depth=2,
                         max_depth=8)
    nat.timing_enable(True)
    nat.timing_read('', reset=True)
    one = sum_z(circuits)
    launches, _ = nat.timing_read('batch', reset=True)
    nat.timing_enable(False)
    assert launches == 1
    nat.call('qg_set_batch_one_launch', 0)
    try:
        per_round = sum_z(circuits)
    finally:
        nat.call('qg_set_batch_one_launch', 1)
    for (n, ops), a, b in zip(circuits, one, per_round):
        want = _oracle_sum_z(n, ops)
        assert abs(a - want) < 2e-5 * n and abs(b - want) < 2e-5 * n, (n, a, b, want)
