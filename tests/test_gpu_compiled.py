"""Compiled circuits (`qgate_gb300.compiled`): one call per circuit and CUDA
graph replay, against the same gates applied one call at a time (the
reference front-end's path, qgate/simulator/rop_executor.py:28-34) and
against the oracle."""
import numpy as np
import pytest

from oracle import statevec as sv
from qgate_gb300 import _native as nat
from qgate_gb300.compiled import CompiledCircuit
from tests.gpu_helpers import (ATOL, apply_ops, fidelity_error, make_gate_type, new_state,
                               random_ops)

pytestmark = pytest.mark.gpu

DTYPES = [np.float64, np.float32]
IDS = ['c128', 'c64']


def _gates(ops):
    return [(make_gate_type(name, args), adj, target, list(ctrls))
            for _, name, args, adj, target, ctrls in ops]


def _state(qs):
    return np.asarray(qs.get_raw()).copy()


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
@pytest.mark.parametrize('graph', [False, True], ids=['direct', 'graph'])
def test_compiled_matches_per_gate_and_oracle(rt, dtype, graph):
    """14 qubits, 300 random (controlled) gates: the compiled run gives the
    per-gate path's state bit for bit (same planning), and the oracle's."""
    n = 14
    rng = np.random.default_rng(7)
    ops = random_ops(rng, n, 300, max_controls=2)
    want = sv.run_ops(n, ops, np.complex128)
    qa = new_state(rt, n, dtype)
    apply_ops(qa, ops)
    ref = _state(qa)
    with CompiledCircuit(dtype, _gates(ops), graph=graph) as circ:
        qb = new_state(rt, n, dtype)
        circ.run(qb)
        got = _state(qb)
        assert circ.stats()[0] == graph
    assert np.array_equal(got, ref)
    assert np.allclose(got, want, atol=ATOL[dtype] * 4)
    qa.delete()
    qb.delete()


@pytest.mark.parametrize('n', [11, 20], ids=['11q', '20q'])
def test_graph_replay_is_deterministic_and_recaptures(rt, n):
    """complex64 with tensor-core stages (20 qubits) and CUDA-core stages (11):
    replays from |0> repeat the first run bit for bit; a fusion-setting
    change, another states buffer and another lane count each re-capture and
    stay correct."""
    rng = np.random.default_rng(n)
    ops = random_ops(rng, n, 400, max_controls=1)
    want = sv.run_ops(n, ops, np.complex128)
    qs = new_state(rt, n, np.float32)
    with CompiledCircuit(np.float32, _gates(ops), graph=True) as circ:
        runs = []
        for _ in range(3):
            qs.processor.reset_qubit_states(qs)
            circ.run(qs)
            runs.append(_state(qs))
        captured, passes = circ.stats()
        assert captured and passes > 0
        assert np.array_equal(runs[0], runs[1]) and np.array_equal(runs[0], runs[2])
        assert fidelity_error(runs[0], want) < 1e-5
        # settings change: re-planned without tensor blocks, then back
        try:
            nat.call('qg_set_tensor_blocks', 0)
            qs.processor.reset_qubit_states(qs)
            circ.run(qs)
            assert fidelity_error(_state(qs), want) < 1e-5
        finally:
            nat.call('qg_set_tensor_blocks', 1)
        # another buffer, and a state with one more lane (|0> on the top lane)
        qb = new_state(rt, n, np.float32)
        circ.run(qb)
        assert np.array_equal(_state(qb), runs[0])
        qc = new_state(rt, n + 1, np.float32)
        circ.run(qc)
        big = _state(qc)
        assert fidelity_error(big[:1 << n], want) < 1e-5
        assert np.max(np.abs(big[1 << n:])) == 0.
        qb.delete()
        qc.delete()
    qs.delete()


def test_graph_after_pending_gates_and_before_observation(rt):
    """Gates queued one call at a time before a graph run are applied first;
    an observation after it sees the whole circuit."""
    n = 16
    rng = np.random.default_rng(3)
    pre = random_ops(rng, n, 50)
    ops = random_ops(rng, n, 200)
    want = sv.run_ops(n, pre + ops, np.complex128)
    qs = new_state(rt, n, np.float64)
    with CompiledCircuit(np.float64, _gates(ops), graph=True) as circ:
        for _ in range(2):
            qs.processor.reset_qubit_states(qs)
            apply_ops(qs, pre)
            circ.run(qs)
            p = qs.processor.calc_probability(qs, 5)
            psi = _state(qs)
            assert np.allclose(psi, want, atol=1e-11)
            assert abs(p - float(np.sum(np.abs(want.reshape(-1, 2, 32)[:, 0, :]) ** 2))) < 1e-11
    qs.delete()


def test_compiled_circuit_errors(rt):
    h = make_gate_type('H', ())
    with pytest.raises(RuntimeError, match='overlapped'):
        CompiledCircuit(np.float32, [(h, False, 2, [2])])
    with pytest.raises(ValueError, match='out of range'):
        CompiledCircuit(np.float32, [(h, False, -1, [])])
    with CompiledCircuit(np.float32, [(h, False, 5, [])], graph=True) as circ:
        small = new_state(rt, 4, np.float32)
        with pytest.raises(ValueError, match='lanes'):
            circ.run(small)
        other = new_state(rt, 8, np.float64)
        with pytest.raises(ValueError, match='precision'):
            circ.run(other)
        small.delete()
        other.delete()
    empty = CompiledCircuit(np.float64, [], graph=True)
    qs = new_state(rt, 3, np.float64)
    empty.run(qs)
    psi = _state(qs)
    assert psi[0] == 1. and np.count_nonzero(psi) == 1
    empty.delete()
    qs.delete()


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_qasm_programs_as_compiled_circuits(rt, dtype):
    """OpenQASM 2.0 programs (qgate_gb300/qasm.py) lowered to compiled
    circuits and run on the engine, against the oracle running the same
    program ops: a 14-qubit QFT of a basis state and a mixed program with
    user gates and multi-controlled standard gates."""
    from qgate_gb300 import qasm
    n = 14
    lines = ['OPENQASM 2.0;', 'include "qelib1.inc";', 'qreg q[%d];' % n, 'x q[3]; x q[9];']
    for i in range(n):
        lines.append('h q[%d];' % i)
        for j in range(i + 1, n):
            lines.append('cu1(pi / %d) q[%d], q[%d];' % (1 << (j - i), j, i))
    mixed = ('OPENQASM 2.0; include "qelib1.inc"; qreg a[7]; qreg b[7];\n'
             'gate lay(t) x, y { ry(t) x; rz(-t / 3) y; cu3(t, t / 2, -t) x, y; }\n'
             'h a; lay(0.7) a, b; ccx a[0], a[1], b[2]; cswap b[0], a[3], b[5];\n'
             'crz(1.3) b[6], a[2]; rzz(0.4) a[4], b[4]; cy a[5], b[1]; sx b;\n')
    for src in ('\n'.join(lines), mixed):
        prog = qasm.parse(src)
        want = sv.initial_state(prog.n_qubits, np.complex128)
        for m, t, c in prog.ops:
            sv.apply_controlled_gate(want, m, list(c), t)
        with prog.compile(dtype, graph=True) as circ:
            qs = new_state(rt, prog.n_qubits, dtype)
            circ.run(qs)
            got = _state(qs)
            qs.delete()
        assert np.allclose(got, want, atol=ATOL[dtype] * 8)


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_qasm_dynamic_programs_shot_by_shot(rt, dtype):
    """OpenQASM programs with mid-circuit measurements, resets and if (run
    shot by shot: compiled gate segments, the runtime's decohere / reset /
    calc_probability between them) against the same programs on the oracle
    runtime with the same uniforms: equal classical registers and states.
    A 12-qubit program interleaving random layers with measure / if / reset
    on a few qubits, and teleportation on every branch."""
    from oracle.runtime import OracleQubitStates
    from qgate_gb300 import qasm
    rng = np.random.default_rng(8)
    n = 12
    lines = ['OPENQASM 2.0;', 'include "qelib1.inc";', 'qreg q[%d];' % n, 'creg c[3];']
    for layer in range(4):
        for q in range(n):
            a, b, g = (float(x) for x in rng.uniform(0, 2 * np.pi, 3))
            lines.append('u3(%r, %r, %r) q[%d];' % (a, b, g, q))
        for k in range(0, n - 1, 2):
            lines.append('cx q[%d], q[%d];' % (k + layer % 2, (k + 1 + layer % 2) % n))
        m = int(rng.integers(n))
        lines.append('measure q[%d] -> c[%d];' % (m, layer % 3))
        lines.append('if (c == %d) h q[%d];' % (layer % 4, (m + 5) % n))
        lines.append('reset q[%d];' % m)
    lines.append('measure q[0] -> c[0]; measure q[1] -> c[1]; measure q[2] -> c[2];')
    progs = ['\n'.join(lines),
             'OPENQASM 2.0; include "qelib1.inc"; qreg q[3]; creg a[1]; creg b[1]; '
             'u3(0.7, 0.4, -1.1) q[0]; h q[1]; cx q[1], q[2]; cx q[0], q[1]; h q[0]; '
             'measure q[0] -> a[0]; measure q[1] -> b[0]; if (b == 1) x q[2]; '
             'if (a == 1) z q[2];']

    def oracle_gates(qs, gates):
        for mat, t, c in gates:
            sv.apply_controlled_gate(qs.psi, mat, list(c), t)

    for src in progs:
        prog = qasm.parse(src)
        assert prog.dynamic
        for trial in range(4):
            u = np.random.default_rng(100 + trial).random(16)
            ref = OracleQubitStates(np.float64)
            ref.processor.initialize_qubit_states(ref, prog.n_qubits)
            ref.processor.reset_qubit_states(ref)
            want_bits = prog.run(ref, randnum=u, gate_runner=oracle_gates)
            qs = new_state(rt, prog.n_qubits, dtype)
            got_bits = prog.run(qs, randnum=u, graph=trial % 2 == 1)
            got = _state(qs)
            qs.delete()
            assert got_bits == want_bits, (src[:40], trial)
            assert np.allclose(got, ref.psi, atol=ATOL[dtype] * 8), (src[:40], trial)
        prog.delete()
