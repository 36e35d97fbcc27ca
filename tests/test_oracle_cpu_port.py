"""The oracle's C port: the cache-blocked circuit runner (cs_run_circuit)
gives exactly the state of one sweep per gate (cs_apply_gate), for random
gates with up to three controls, in both precisions and for several pass
sizes, and the complex128 result agrees with the numpy restatement
(oracle/statevec.py) to FP64 rounding."""
import numpy as np
import pytest

from oracle import cpu_port, statevec as sv


def _gates(rng, n, count):
    out = []
    for _ in range(count):
        q = rng.permutation(n)
        nc = int(rng.integers(0, 4))
        name, args = ('U', tuple(rng.uniform(0, 2 * np.pi, 3))) if rng.random() < 0.7 else ('X', ())
        out.append((name, args, int(q[0]), tuple(int(x) for x in q[1:1 + nc])))
    return out


@pytest.mark.parametrize('n, max_lanes', [(6, 5), (12, 8), (15, 10), (16, 14)])
@pytest.mark.parametrize('dtype', [np.complex128, np.complex64])
def test_blocked_passes_equal_per_gate_sweeps(n, max_lanes, dtype):
    rng = np.random.default_rng(n * 31 + max_lanes)
    ops = _gates(rng, n, 120)
    gates = [(sv.gate_matrix(nm, a), t, c) for nm, a, t, c in ops]
    a = cpu_port.State(n, dtype)
    for m, t, c in gates:
        a.apply(m, t, c)
    b = cpu_port.State(n, dtype)
    passes = b.run(gates, max_lanes)
    assert 1 <= passes <= len(gates)
    assert np.array_equal(a.psi, b.psi)
    if dtype == np.complex128:
        want = sv.run_ops(n, [('g', nm, a_, False, t, c) for nm, a_, t, c in ops], np.complex128)
        assert np.max(np.abs(b.psi - want)) < 1e-13


def test_prefix_cdf_and_sampling_match_the_pool_rule():
    rng = np.random.default_rng(5)
    p = rng.random(1 << 10)
    p /= p.sum()
    cdf, total = cpu_port.prefix_cdf(p)
    assert abs(total - 1.) < 1e-12 and abs(cdf[-1] - 1.) < 1e-15
    u = rng.random(5000)
    got = cpu_port.sample_cdf(cdf, u)
    want = np.minimum(np.searchsorted(cdf, u, side='right'), len(p) - 1)
    assert np.array_equal(got, want)
