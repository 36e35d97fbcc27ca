"""The headline and large configurations against independent answers.

30 qubits (the random U3 + CX circuit, depth 20: U3 angles from
default_rng(10), CX matchings from default_rng(11)): the engine's complex64
and complex128 runs through the plugin API against the oracle's C port of the
reference CPU runtime in complex128 on the host (oracle/cpu_statevec.c,
cs_run_circuit: per-pair arithmetic of qgate/simulator/src/
CPUQubitProcessor.cpp:307-362, cache-blocked passes, the same result as one
sweep per gate).  Stated per precision: the fidelity error
|1 - |<psi_oracle|psi_engine>|| and the largest probability error.  Then 1e7
uniforms from default_rng(12) through the engine's complex64 sampling pool and
through the oracle's FP64 pool (qgate/simulator/src/CPUSamplingPool.cpp:8-81):
indices must agree except where u lies within tau of a boundary of the
oracle's CDF, tau = max_k |cdf_engine[k] - cdf_oracle[k]| (cdf_engine from the
engine's complex64 amplitudes, squared and summed in FP64).

34 qubits (the QFT without final swaps of a basis state, X on qubit i iff
default_rng(41).random() < 0.5): the analytic answer.  Every amplitude has
modulus 2^-17, so prob[k] = 2^-34, Pr(q = 0) = 1/2 for every qubit, the CDF
is (k + 1) / 2^34 and u samples floor(u 2^34).  1e8 uniforms from
default_rng(42) through the engine's pool must land within tau 2^34 + 1
indices of floor(u 2^34), tau being the largest deviation of the engine's
CDF (prefix sums of its probabilities in FP64) from (k + 1) / 2^34.

Tolerances: complex64 fidelity error < 1e-5 and probability error < 1e-7 per
amplitude (relative to 2^-34 for the QFT: 1e-5); complex128 fidelity error
< 1e-11, probability error < 1e-13; Pr(q = 0) within 5e-6 (complex64)."""
import math

import numpy as np
import pytest

from tests.gpu_helpers import Lane, abs2

pytestmark = pytest.mark.gpu

N1, DEPTH = 30, 20


def _c1_gates():
    """[(name, args, target, controls)] of the 30-qubit random circuit."""
    ang = np.random.default_rng(10).uniform(0, 2 * math.pi, (DEPTH, N1, 3))
    prng = np.random.default_rng(11)
    ops = []
    for layer in range(DEPTH):
        ops += [('U', tuple(float(a) for a in ang[layer, q]), q, ()) for q in range(N1)]
        p = prng.permutation(N1)
        ops += [('X', (), int(p[2 * k + 1]), (int(p[2 * k]),)) for k in range(N1 // 2)]
    return ops


def _run_engine(rt, n, ops, dtype):
    from qgate_gb300.circuit import gate_type
    qs = rt.create_qubit_states(dtype)
    proc = qs.processor
    proc.initialize_qubit_states(qs, n)
    proc.reset_qubit_states(qs)
    for name, args, t, c in ops:
        g = gate_type(name, *args)
        if c:
            proc.apply_controlled_gate(g, False, qs, list(c), t)
        else:
            proc.apply_gate(g, False, qs, t)
    proc.synchronize()
    return qs


def _compare(ref, got, step=1 << 26):
    """(fidelity error, max probability error) of `got` against `ref`,
    summed in FP64 in slices."""
    ov = 0j
    perr = 0.
    for i in range(0, ref.size, step):
        a = ref[i:i + step]
        b = got[i:i + step].astype(np.complex128)
        ov += np.vdot(a, b)
        perr = max(perr, float(np.max(np.abs(np.abs(a) ** 2 - np.abs(b) ** 2))))
    return abs(1. - abs(ov)), perr


@pytest.fixture(scope='module')
def c1_oracle():
    """The oracle's complex128 state of the 30-qubit circuit (16 GiB, host)."""
    from oracle import cpu_port, statevec as sv
    ops = _c1_gates()
    mats = {}
    gates = []
    for name, args, t, c in ops:
        if (name, args) not in mats:
            mats[(name, args)] = sv.gate_matrix(name, args)
        gates.append((mats[(name, args)], t, c))
    st = cpu_port.State(N1, np.complex128)
    st.run(gates, 14)
    return ops, st


def test_c1_30q_complex128_against_fp64_oracle(rt, c1_oracle):
    ops, st = c1_oracle
    qs = _run_engine(rt, N1, ops, np.float64)
    got = qs.get_raw()
    qs.delete()
    ferr, perr = _compare(st.psi, got)
    del got
    print('c1 30q complex128: fidelity error %.3e, max probability error %.3e' % (ferr, perr))
    assert ferr < 1e-11 and perr < 1e-13, (ferr, perr)


def test_c1_30q_complex64_and_samples_against_fp64_oracle(rt, c1_oracle):
    from oracle import cpu_port
    ops, st = c1_oracle
    qs = _run_engine(rt, N1, ops, np.float32)
    got = qs.get_raw()
    ferr, perr = _compare(st.psi, got)
    print('c1 30q complex64: fidelity error %.3e, max probability error %.3e' % (ferr, perr))
    assert ferr < 1e-5 and perr < 1e-7, (ferr, perr)

    u = np.random.default_rng(12).random(10_000_000)
    getter = rt.create_qubits_states_getter(np.float32)
    pool = getter.create_sampling_pool(list(range(N1)), N1, 0,
                                       [(qs, [Lane(l, l) for l in range(N1)])], [])
    idx_e = np.asarray(pool.sample(len(u), u).intarray)
    pool.delete()
    qs.delete()

    cdf_r, total = cpu_port.prefix_cdf(st.probabilities(), copy=False)
    assert abs(total - 1.) < 1e-12
    idx_r = cpu_port.sample_cdf(cdf_r, u)
    # the engine's CDF from its own amplitudes, in FP64
    p_e = got.real.astype(np.float64) ** 2 + got.imag.astype(np.float64) ** 2
    del got
    cdf_e = np.cumsum(p_e)
    cdf_e /= cdf_e[-1]
    del p_e
    tau = float(np.max(np.abs(cdf_e - cdf_r))) + 1e-15
    del cdf_e
    diff = idx_e != idx_r
    hi = cdf_r[idx_r]
    lo = np.where(idx_r > 0, cdf_r[np.maximum(idx_r - 1, 0)], 0.)
    near = (np.abs(u - hi) <= tau) | (np.abs(u - lo) <= tau)
    print('c1 30q samples: tau %.3e, %d of %d differ, %d near a boundary'
          % (tau, int(diff.sum()), len(u), int(near.sum())))
    assert tau < 1e-6, tau
    assert not np.any(diff & ~near), int(np.sum(diff & ~near))


def test_qft_34q_against_the_analytic_answer(rt):
    n = 34
    N = 1 << n
    rng = np.random.default_rng(41)
    ops = [('X', (), q, ()) for q in range(n) if rng.random() < 0.5]
    for i in range(n):
        ops.append(('H', (), i, ()))
        for j in range(i + 1, n):
            ops.append(('U1', (math.pi / (1 << (j - i)),), i, (j,)))
    qs = _run_engine(rt, n, ops, np.float32)
    assert abs(qs.processor.calc_norm(qs) - 1.) < 1e-5
    pr = np.array([qs.processor.calc_probability(qs, q) for q in range(n)])
    assert np.max(np.abs(pr - 0.5)) < 5e-6, pr

    # probability vector in 2^30-entry chunks: deviation from 2^-n and the
    # engine's CDF against (k + 1) / 2^n
    getter = rt.create_qubits_states_getter(np.float32)
    lanes = [(qs, [Lane(l, l) for l in range(n)])]
    chunk = min(N, 1 << 30)
    buf = np.empty(chunk, np.float32)
    carry, dev_p, dev_cdf = 0., 0., 0.
    for start in range(0, N, chunk):
        getter.get_states(buf, 0, abs2, lanes, [], chunk, start, 1)
        p = buf.astype(np.float64)
        dev_p = max(dev_p, float(np.max(np.abs(p * N - 1.))))
        c = np.cumsum(p)
        c += carry
        carry = float(c[-1])
        k1 = np.arange(start + 1, start + chunk + 1, dtype=np.float64)
        dev_cdf = max(dev_cdf, float(np.max(np.abs(c - k1 / N))))
        del p, c, k1
    del buf
    total = carry
    tau = dev_cdf + abs(total - 1.) + 1e-12
    print('qft %dq: max |prob 2^n - 1| %.3e, max |Pr - 1/2| %.3e, cdf deviation %.3e '
          '(%.1f entries)' % (n, dev_p, float(np.max(np.abs(pr - 0.5))), tau, tau * N))
    assert dev_p < 1e-5, dev_p

    u = np.random.default_rng(42).random(100_000_000)
    pool = getter.create_sampling_pool(list(range(n)), n, 0, lanes, [])
    got = np.asarray(pool.sample(len(u), u).intarray)
    pool.delete()
    qs.delete()
    want = np.floor(u * N).astype(np.int64)
    off = np.abs(got - want)
    bound = int(math.ceil(tau * N)) + 1
    print('qft %dq samples: %d exact of %d, largest index offset %d (bound %d)'
          % (n, int(np.sum(off == 0)), len(u), int(off.max()), bound))
    assert int(off.max()) <= bound, (int(off.max()), bound)
