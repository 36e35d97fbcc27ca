"""The reference's CPU-runnable case at its own size: a 20-qubit QFT without
final swaps on |x> (X on qubit i iff default_rng(0).random() < 0.5, in qubit
order), then the full probability vector, Pr(q_i = 0) for every qubit and
1e6 samples from default_rng(1) uniforms, through the plugin API.

Oracle: the analytic result.  The QFT of a basis state has every amplitude
of modulus 2^-n/2, so prob[k] = 2^-20 exactly, every Pr(q = 0) = 1/2, the
CDF is (k + 1) / 2^20 and a uniform u samples index floor(u * 2^20) - the
same answers the reference's complex128 CPU runtime gives (its QFT traces at
8 and 14 qubits are replayed bit-for-bit elsewhere).  Sampled indices must
match except where u lies within tau of a CDF boundary, tau = twice the
largest deviation of the CDF of the engine's probabilities from
(k + 1) / 2^20.  Tolerances: complex128 1e-12 on Pr, 1e-12 relative on
probabilities; complex64 1e-6 / 1e-5."""
import numpy as np
import pytest

from tests.gpu_helpers import Lane, abs2, apply_ops, new_state

pytestmark = pytest.mark.gpu

N = 20


def _c0_ops():
    rng = np.random.default_rng(0)
    ops = [('g', 'X', (), False, q, ()) for q in range(N) if rng.random() < 0.5]
    for i in range(N):
        ops.append(('g', 'H', (), False, i, ()))
        for j in range(i + 1, N):
            ops.append(('g', 'U1', (np.pi / (1 << (j - i)),), False, i, (j,)))
    return ops


@pytest.mark.parametrize('dtype', [np.float64, np.float32], ids=['c128', 'c64'])
def test_c0_qft20_prob_pauli_samples(rt, dtype):
    qs = new_state(rt, N, dtype)
    apply_ops(qs, _c0_ops())
    p_tol, rel_tol = (1e-12, 1e-12) if dtype == np.float64 else (1e-6, 1e-5)
    for q in range(N):
        assert abs(qs.processor.calc_probability(qs, q) - 0.5) < p_tol, q
    getter = rt.create_qubits_states_getter(dtype)
    lanes = [(qs, [Lane(l, l) for l in range(N)])]
    probs = np.empty(1 << N, dtype)
    getter.get_states(probs, 0, abs2, lanes, [], 1 << N, 0, 1)
    dev = np.max(np.abs(probs.astype(np.float64) * (1 << N) - 1.))
    assert dev < rel_tol, dev
    u = np.random.default_rng(1).random(1_000_000)
    pool = getter.create_sampling_pool(list(range(N)), N, 0, lanes, [])
    got = np.asarray(pool.sample(len(u), u).intarray)
    pool.delete()
    x = u * (1 << N)
    want = np.floor(x).astype(np.int64)
    # tau: the engine's CDF deviation from (k + 1) / 2^N (from the
    # probabilities it returned), doubled, in index units
    cdf = np.cumsum(probs.astype(np.float64))
    cdf /= cdf[-1]
    tau = 2. * (np.max(np.abs(cdf - np.arange(1, (1 << N) + 1) / (1 << N))) + 1e-12) * (1 << N)
    near = np.abs(x - np.round(x)) <= tau
    assert np.array_equal(got[~near], want[~near])
    assert np.mean(near) < 0.05, (tau, np.mean(near))
    qs.delete()
