"""The bench's synthetic workloads match their specification (CPU only):
the random U3 + CX circuit (angles from default_rng(10), CX matchings from
default_rng(11), per layer), its unfused gate-pass byte count, and the QFT
case (X preparation from default_rng(seed), then H and the controlled-U1
ladder, no swaps), which the oracle turns into the uniform distribution."""
import math

import numpy as np

import bench
from oracle import statevec as sv


def test_random_circuit_layers_follow_the_seeds():
    n, depth = 30, 20
    ops = bench.circuit(n, depth)
    assert len(ops) == depth * (n + n // 2)
    ang = np.random.default_rng(10).uniform(0, 2 * math.pi, (depth, n, 3))
    prng = np.random.default_rng(11)
    k = 0
    for layer in range(depth):
        for q in range(n):
            name, args, target, ctrls = ops[k]
            assert (name, target, ctrls) == ('U', q, ())
            assert np.array_equal(np.asarray(args), ang[layer, q])
            k += 1
        p = prng.permutation(n)
        for j in range(n // 2):
            assert ops[k] == ('X', (), int(p[2 * j + 1]), (int(p[2 * j]),))
            k += 1


def test_gate_pass_bytes():
    n = 30
    ops = bench.circuit(n, 20)
    want = 20 * (30 * 2 * (1 << n) * 8 + 15 * 2 * (1 << (n - 1)) * 8)
    assert bench.gate_pass_bytes(n, ops, 8) == want


def test_qft_case_gives_uniform_probabilities():
    n = 10
    ops = bench.qft_ops(n, 0)
    rng = np.random.default_rng(0)
    xs = [q for q in range(n) if rng.random() < 0.5]
    assert [o[2] for o in ops[:len(xs)] if o[0] == 'X'] == xs
    assert sum(1 for o in ops if o[0] == 'U1') == n * (n - 1) // 2
    psi = sv.run_ops(n, [('g', nm, a, False, t, c) for nm, a, t, c in ops])
    assert np.allclose(np.abs(psi) ** 2, 1. / (1 << n), atol=1e-12)


def test_reference_arm_line_carries_the_shared_config(capsys):
    """The reference arm's line (the oracle's C port on host cores) reports
    the same `config` object as the GPU arm's: the workload and the metric's
    definition, no measured figures."""
    import argparse
    import json
    args = argparse.Namespace(qubits=12, depth=20, dtype='c64', steps=1, warmup=0, gpus=1,
                              ref_gates=45, samples=1000)
    bench.run_reference(args)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line['impl'] == 'reference'
    assert line['config'] == bench.config_block(args)
    assert line['metric'] == bench.METRIC and line['value'] > 0
    assert line['e2e']['h2d_bytes_per_step'] == 0 and line['e2e']['d2h_bytes_per_step'] == 0
    assert line['cpu_baseline']['kind'] == 'port' and line['cpu_baseline']['cores'] >= 1
    obs = line['cpu_baseline']['observations']
    assert obs['sample']['samples'] == 1000 and obs['sample']['samples_per_s'] > 0
    assert all(obs[k]['gbs'] > 0 for k in ('prob', 'probability_vector', 'pool_prefix_sums'))


def test_cpu_leg_helpers():
    """The GPU arm's cpu_baseline leg: the port's gate rate on the circuit's
    first gates and its observation timings on the same host state."""
    ops = bench.circuit(14, 20)
    gbs, done, dt, threads, st = bench.cpu_port_gate_rate(14, ops, 8, 0.05)
    assert gbs > 0 and 1 <= done <= len(ops) and threads >= 1 and st.n == 14
    obs = bench.cpu_port_observations(st, 5000)
    assert obs['sample']['samples'] == 5000 and obs['threads'] == threads
