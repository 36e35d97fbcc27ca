"""OpenQASM 2.0 front-end (qgate_gb300/qasm.py) on the CPU: parsing,
broadcasting, user gates and expressions; the standard gates' matrices
against their definitions; whole programs run by the oracle; and the errors
for what a compiled circuit cannot run."""
import math

import numpy as np
import pytest

from oracle import statevec as sv
from qgate_gb300 import qasm


def run(prog, psi=None):
    """The program's ops applied by the oracle (lane i = qubit i)."""
    if psi is None:
        psi = sv.initial_state(prog.n_qubits, np.complex128)
    for m, t, c in prog.ops:
        sv.apply_controlled_gate(psi, m, list(c), t)
    return psi


def expm_pauli(theta, P):
    """exp(-i theta P / 2) for a Pauli matrix P."""
    return math.cos(theta / 2) * np.eye(2) - 1j * math.sin(theta / 2) * P


X = np.array([[0, 1], [1, 0]], complex)
Y = np.array([[0, -1j], [1j, 0]], complex)
Z = np.diag([1, -1]).astype(complex)


def one(name_args):
    p = qasm.parse('OPENQASM 2.0; include "qelib1.inc"; qreg q[1]; %s q[0];' % name_args)
    assert len(p.ops) == 1
    return p.ops[0][0]


def test_standard_one_qubit_matrices():
    h = np.array([[1, 1], [1, -1]]) / math.sqrt(2)
    assert np.allclose(one('h'), h)
    assert np.allclose(one('u2(0, pi)'), h)
    assert np.allclose(one('x'), X) and np.allclose(one('u3(pi, 0, pi)'), X)
    assert np.allclose(one('y'), Y) and np.allclose(one('z'), Z)
    for t in (0.3, -1.7, 2.9):
        assert np.allclose(one('rx(%r)' % t), expm_pauli(t, X))
        assert np.allclose(one('ry(%r)' % t), expm_pauli(t, Y))
        assert np.allclose(one('rz(%r)' % t), np.diag([1, np.exp(1j * t)]))
        assert np.allclose(one('u1(%r)' % t), np.diag([1, np.exp(1j * t)]))
    assert np.allclose(one('s'), np.diag([1, 1j])) and np.allclose(one('sdg'), np.diag([1, -1j]))
    assert np.allclose(one('t'), np.diag([1, np.exp(0.25j * math.pi)]))
    assert np.allclose(one('sx') @ one('sx'), -1j * X)  # sqrt(X) up to phase
    u = one('u3(0.4, 1.1, -0.7)')
    assert np.allclose(u.conj().T @ u, np.eye(2))
    assert np.allclose(u, [[math.cos(0.2), -np.exp(-0.7j) * math.sin(0.2)],
                           [np.exp(1.1j) * math.sin(0.2), np.exp(0.4j) * math.cos(0.2)]])


def test_u_gates_differ_from_the_reference_translation_by_a_global_phase():
    """The reference translates U / u3 / u2 to qgate's U3 / U2 (the oracle's
    'U' / 'U2' matrices, pinned to matrices recorded from the reference),
    which carry an extra global phase exp(-i (phi + lambda) / 2)."""
    for t, p, l in ((0.4, 1.1, -0.7), (2.9, -0.3, 1.6), (-1.2, 0.0, 2.2)):
        want = np.asarray(sv.gate_matrix('U', (t, p, l)))
        phase = np.exp(-0.5j * (p + l))
        assert np.allclose(want, phase * one('U(%r, %r, %r)' % (t, p, l)), atol=1e-14)
        assert np.allclose(want, phase * one('u3(%r, %r, %r)' % (t, p, l)), atol=1e-14)
        assert np.allclose(np.asarray(sv.gate_matrix('U2', (p, l))),
                           phase * one('u2(%r, %r)' % (p, l)), atol=1e-14)


def test_expression_power_rules():
    # '^' is a power, right-associative, binding tighter than unary minus
    assert np.allclose(one('u1(-2^2)'), np.diag([1, np.exp(-4j)]))
    assert np.allclose(one('u1(2^3^2 / 256)'), np.diag([1, np.exp(2j)]))
    assert np.allclose(one('u1((-2)^2)'), np.diag([1, np.exp(4j)]))
    assert np.allclose(one('u1(2 * 3^2 - 1)'), np.diag([1, np.exp(17j)]))


def test_parse_registers_broadcast_user_gates_expressions():
    src = """
    OPENQASM 2.0;
    include "qelib1.inc";
    // a comment
    qreg a[2]; qreg b[2];
    creg c[4];
    gate mine(t, p) x, y { rz(t / 2) x; cx x, y; U(p, 0, -p) y; }
    h a;                       // broadcast over a
    cx a, b;                   // pairwise: a[0]->b[0], a[1]->b[1]
    mine(pi^2 / 4, -sin(pi/6)) a[1], b[0];
    barrier a, b;
    measure a -> c[0:0];
    """
    with pytest.raises(qasm.QasmError):
        qasm.parse(src)  # c[0:0] is not OpenQASM
    p = qasm.parse(src.replace('measure a -> c[0:0];',
                               'measure a[0] -> c[1]; measure b[1] -> c[2];'))
    assert p.n_qubits == 4 and p.n_clbits == 4
    assert p.measurements == [(0, 1), (3, 2)]
    assert p.qregs == {'a': (0, 2), 'b': (2, 2)}
    kinds = [(t, c) for _, t, c in p.ops]
    assert kinds[:4] == [(0, ()), (1, ()), (2, (0,)), (3, (1,))]
    assert kinds[4:] == [(1, ()), (2, (1,)), (2, ())]
    assert np.allclose(p.ops[4][0], np.diag([1, np.exp(1j * math.pi ** 2 / 8)]))
    assert np.allclose(p.ops[6][0], qasm._u(-0.5, 0, 0.5))
    with pytest.raises(qasm.QasmError, match='different sizes'):
        qasm.parse('OPENQASM 2.0; qreg a[2]; qreg b[2]; creg c[3]; measure a -> c;')


def test_programs_on_the_oracle():
    n = 6
    lines = ['OPENQASM 2.0;', 'include "qelib1.inc";', 'qreg q[%d];' % n, 'x q[1]; x q[4];']
    for i in range(n):
        lines.append('h q[%d];' % i)
        for j in range(i + 1, n):
            lines.append('cu1(pi / %d) q[%d], q[%d];' % (1 << (j - i), j, i))
    psi = run(qasm.parse('\n'.join(lines)))
    assert np.allclose(np.abs(psi) ** 2, 1. / (1 << n))  # QFT of a basis state
    ghz = run(qasm.parse('OPENQASM 2.0; include "qelib1.inc"; qreg q[3]; h q[0]; '
                         'cx q[0], q[1]; cx q[1], q[2];'))
    want = np.zeros(8, complex)
    want[0] = want[7] = 1 / math.sqrt(2)
    assert np.allclose(ghz, want)
    sw = run(qasm.parse('OPENQASM 2.0; include "qelib1.inc"; qreg q[2]; x q[0]; '
                        'swap q[0], q[1];'))
    assert np.allclose(sw, [0, 0, 1, 0])
    for bits in range(8):  # Toffoli and Fredkin truth tables
        prep = ''.join('x q[%d]; ' % k for k in range(3) if bits >> k & 1)
        out = run(qasm.parse('OPENQASM 2.0; include "qelib1.inc"; qreg q[3]; %s'
                             'ccx q[0], q[1], q[2];' % prep))
        assert np.argmax(np.abs(out)) == (bits ^ 4 if bits & 3 == 3 else bits)
        out = run(qasm.parse('OPENQASM 2.0; include "qelib1.inc"; qreg q[3]; %s'
                             'cswap q[0], q[1], q[2];' % prep))
        sw = bits
        if bits & 1:
            b1, b2 = bits >> 1 & 1, bits >> 2 & 1
            sw = 1 | (b2 << 1) | (b1 << 2)
        assert np.argmax(np.abs(out)) == sw


@pytest.mark.parametrize('gate, target_op', [
    ('cy', Y), ('cz', Z), ('ch', np.array([[1, 1], [1, -1]]) / math.sqrt(2)),
    ('crz(0.9)', np.diag([np.exp(-0.45j), np.exp(0.45j)])),
    ('cu1(0.9)', np.diag([1, np.exp(0.9j)])),
    ('cu3(0.4, 1.1, -0.7)', qasm._u(0.4, 1.1, -0.7)),
    ('crx(0.8)', expm_pauli(0.8, X)), ('cry(0.8)', expm_pauli(0.8, Y))])
def test_controlled_gates_act_on_the_target_only_when_the_control_is_set(gate, target_op):
    rng = np.random.default_rng(3)
    v = rng.standard_normal(2) + 1j * rng.standard_normal(2)
    v /= np.linalg.norm(v)
    for ctl in (0, 1):
        psi = np.zeros(4, complex)  # control = qubit 0, target = qubit 1
        psi[ctl] = v[0]
        psi[ctl | 2] = v[1]
        out = run(qasm.parse('OPENQASM 2.0; include "qelib1.inc"; qreg q[2]; %s q[0], q[1];'
                             % gate), psi)
        w = target_op @ v if ctl else v
        assert np.allclose([out[ctl], out[ctl | 2]], w)


def test_rzz_and_user_gate_nesting():
    p = qasm.parse('OPENQASM 2.0; include "qelib1.inc"; qreg q[2]; '
                   'gate g(a) x, y { rzz(a) x, y; } gate g2(b) u, w { g(2*b) w, u; } '
                   'h q; g2(0.35) q[0], q[1];')
    psi = run(p)
    ph = np.exp(1j * 0.7 * np.array([0, 1, 1, 0]))  # diag over (q1 q0) = 00, 01, 10, 11
    assert np.allclose(psi, 0.5 * ph)


@pytest.mark.parametrize('src, msg', [
    ('OPENQASM 3.0; qreg q[1];', 'OpenQASM 2.0'),
    ('OPENQASM 2.0; qreg q[1]; h q[0];', 'qelib1'),
    ('OPENQASM 2.0; include "qelib1.inc"; qreg q[1]; cx q[0];', 'takes 0 parameters and 2'),
    ('OPENQASM 2.0; include "qelib1.inc"; qreg q[2]; cx q[0], q[0];', 'twice'),
    ('OPENQASM 2.0; include "qelib1.inc"; qreg q[2]; qreg r[3]; cx q, r;', 'different sizes'),
    ('OPENQASM 2.0; qreg q[1]; creg c[1]; if (d == 1) U(0, 0, 0) q[0];', 'unknown creg'),
    ('OPENQASM 2.0; qreg q[1]; creg c[1]; if (c == 1) barrier q;', 'cannot follow if'),
    ('OPENQASM 2.0; opaque g q;', 'opaque'),
    ('OPENQASM 2.0; qreg q[1]; U(1/0, 0, 0) q[0];', 'division by zero'),
    ('OPENQASM 2.0; qreg q[1]; gate g x { U(t, 0, 0) x; } g q[0];', 'unknown parameter'),
    ('OPENQASM 2.0; qreg q[2]; U(0, 0, 0) q[2];', 'out of range'),
    ('OPENQASM 2.0; qreg q[1]; qreg q[1];', 'declared twice'),
    ('OPENQASM 2.0; qreg q[1]; gate g x { g x; } g q[0];', 'recursively'),
])
def test_errors(src, msg):
    with pytest.raises(qasm.QasmError, match=msg):
        qasm.parse(src)


def test_exponential_expansion_is_stopped(monkeypatch):
    """User gates that each call the previous one twice double the gate count
    per level: the parser stops at its gate cap with a parse error."""
    monkeypatch.setattr(qasm, 'MAX_OPS', 1000)
    src = 'OPENQASM 2.0; qreg q[1]; gate g0 x { U(0.1, 0, 0) x; } '
    for k in range(1, 16):
        src += 'gate g%d x { g%d x; g%d x; } ' % (k, k - 1, k - 1)
    with pytest.raises(qasm.QasmError, match='more than 1000 gates'):
        qasm.parse(src + 'g15 q[0];')


def test_reset_of_a_fresh_qubit_and_terminal_measurements():
    p = qasm.parse('OPENQASM 2.0; include "qelib1.inc"; qreg q[2]; creg c[2]; reset q; '
                   'h q[0]; cx q[0], q[1]; barrier q; measure q -> c;')
    assert len(p.ops) == 2 and p.measurements == [(0, 0), (1, 1)]


def test_compiled_circuit_from_a_program():
    """The gate table builds on the host (no device work until it runs)."""
    p = qasm.parse('OPENQASM 2.0; include "qelib1.inc"; qreg q[3]; h q; ccx q[0], q[1], q[2];'
                   'cu3(0.1, 0.2, 0.3) q[2], q[0];')
    c = p.compile(np.float64, graph=False)
    assert c.n_gates == 5
    c.delete()


class _FakeQstates:
    """Stands in for a states object: the oracle's state vector."""

    def __init__(self, psi):
        self.psi = psi

        class P:
            dtype = np.float64
        self.processor = P()

    def get_n_lanes(self):
        return int(self.psi.size).bit_length() - 1


class _FakeRuntime:
    """The runtime calls QasmProgram.sample makes, answered by the oracle:
    the marginal over the pool lanes (hidden lanes summed out) and its FP64
    sampling pool."""

    def create_qubits_states_getter(self, dtype):
        return self

    def create_sampling_pool(self, ordering, n_lanes, n_hidden, lane_trans, empty):
        (qs, lanes), = lane_trans
        assert empty == [] and n_lanes + n_hidden == qs.get_n_lanes()
        h = n_lanes
        table = []
        for ln in lanes:
            if ln.external == -1:
                table.append(h)
                h += 1
            else:
                table.append(ln.external)
        prob = sv.marginal_probabilities([(qs.psi, table)], n_lanes, n_hidden)
        pool = sv.SamplingPool(prob)

        class Pool:
            def sample(self, shots, u):
                class Obs:
                    intarray = pool.sample(u[:shots])
                return Obs()

            def delete(self):
                pass
        return Pool()


def test_sample_maps_measured_lanes_to_classical_bits():
    src = ('OPENQASM 2.0; include "qelib1.inc"; qreg q[4]; creg c[3]; h q[2]; '
           'cx q[2], q[0]; x q[3]; measure q[0] -> c[2]; measure q[2] -> c[0]; '
           'measure q[3] -> c[1]; measure q[1] -> c[1];')
    prog = qasm.parse(src)
    assert prog.measurements == [(2, 0), (1, 1), (0, 2)]  # c[1] keeps the later q[1]
    qs = _FakeQstates(run(prog))
    u = np.random.default_rng(4).random(4000)
    out = prog.sample(_FakeRuntime(), qs, len(u), u)
    # q[0] = q[2] (GHZ pair) -> c[2] = c[0]; q[1] = 0 -> c[1] = 0
    assert set(np.unique(out)) == {0b000, 0b101}
    assert 0.45 < np.mean(out == 0b101) < 0.55
    with pytest.raises(qasm.QasmError, match='measures nothing'):
        qasm.parse('OPENQASM 2.0; qreg q[1];').sample(_FakeRuntime(), qs, 1)


# ------------------------------------------------------------------ dynamic programs

class _OracleStates:
    """A states object of the oracle runtime (oracle/runtime.py) with n lanes
    in |0...0>."""

    def __new__(cls, n):
        from oracle.runtime import OracleQubitStates
        qs = OracleQubitStates(np.float64)
        qs.processor.initialize_qubit_states(qs, n)
        qs.processor.reset_qubit_states(qs)
        return qs


def _oracle_gates(qs, gates):
    for m, t, c in gates:
        if c:
            sv.apply_controlled_gate(qs.psi, m, list(c), t)
        else:
            sv.apply_gate(qs.psi, m, t)


TELEPORT = ('OPENQASM 2.0; include "qelib1.inc"; qreg q[3]; creg a[1]; creg b[1]; '
            'u3(0.7, 0.4, -1.1) q[0]; h q[1]; cx q[1], q[2]; cx q[0], q[1]; h q[0]; '
            'measure q[0] -> a[0]; measure q[1] -> b[0]; '
            'if (b == 1) x q[2]; if (a == 1) z q[2];')


def test_dynamic_program_items():
    p = qasm.parse(TELEPORT)
    assert p.dynamic
    kinds = [it[0] for it in p.items]
    assert kinds == ['g'] * 5 + ['m', 'm', 'if', 'if']
    assert p.items[7][1:4] == (1, 1, 1) and p.items[7][4][0][0] == 'g'
    with pytest.raises(qasm.QasmError, match='run it shot by shot'):
        p.compile()
    static = qasm.parse('OPENQASM 2.0; include "qelib1.inc"; qreg q[2]; creg c[2]; reset q; '
                        'h q[0]; measure q -> c;')
    assert not static.dynamic


@pytest.mark.parametrize('u', [(0.1, 0.1), (0.1, 0.9), (0.9, 0.1), (0.9, 0.9)])
def test_teleportation_every_branch(u):
    """Whatever the two outcomes, q[2] ends in the state q[0] started in."""
    p = qasm.parse(TELEPORT)
    qs = _OracleStates(3)
    bits = p.run(qs, randnum=list(u), gate_runner=_oracle_gates)
    psi = qs.psi.reshape(2, 2, 2)  # [q2, q1, q0]
    a, b = bits & 1, bits >> 1 & 1
    assert (qs.get_lane_state(0), qs.get_lane_state(1)) == (a, b)
    q2 = psi[:, b, a]
    want = qasm._u(0.7, 0.4, -1.1) @ np.array([1, 0])
    assert abs(abs(np.vdot(want, q2)) - 1.) < 1e-12


def test_measurement_follows_the_reference_rule():
    """outcome 0 iff u < Pr(q = 0); the state collapses; a reset of a qubit
    measured 1 brings it back to |0>."""
    p = qasm.parse('OPENQASM 2.0; include "qelib1.inc"; qreg q[1]; creg c[1]; '
                   'ry(1.0) q[0]; measure q[0] -> c[0]; reset q[0]; measure q[0] -> c[0];')
    p0 = math.cos(0.5) ** 2
    for u, first in ((p0 - 1e-9, 0), (p0 + 1e-9, 1)):
        qs = _OracleStates(1)
        bits = []
        orig = qs.processor.decohere

        def record(v, prob, q, lane, orig=orig):
            bits.append(v)
            return orig(v, prob, q, lane)
        qs.processor.decohere = record
        out = p.run(qs, randnum=[u, 0.5], gate_runner=_oracle_gates)
        assert bits == [first, 0] and out == 0
        assert np.allclose(qs.psi, [1, 0])


def test_reset_needs_a_measured_or_fresh_qubit():
    ok = qasm.parse('OPENQASM 2.0; include "qelib1.inc"; qreg q[2]; creg c[1]; reset q[1]; '
                    'x q[0]; measure q[0] -> c[0]; reset q[0]; reset q[0];')
    qs = _OracleStates(2)
    assert ok.run(qs, randnum=[0.5], gate_runner=_oracle_gates) == 1
    assert np.allclose(qs.psi, [1, 0, 0, 0])
    bad = qasm.parse('OPENQASM 2.0; include "qelib1.inc"; qreg q[1]; h q[0]; reset q[0];')
    with pytest.raises(RuntimeError, match='not measured'):
        bad.run(_OracleStates(1), gate_runner=_oracle_gates)
    # a gate on a measured qubit makes it unmeasured again
    stale = qasm.parse('OPENQASM 2.0; include "qelib1.inc"; qreg q[1]; creg c[1]; x q[0]; '
                       'measure q[0] -> c[0]; h q[0]; reset q[0];')
    with pytest.raises(RuntimeError, match='not measured'):
        stale.run(_OracleStates(1), randnum=[0.5], gate_runner=_oracle_gates)


def test_if_compares_the_whole_register():
    src = ('OPENQASM 2.0; include "qelib1.inc"; qreg q[3]; creg c[2]; x q[1]; '
           'measure q[0] -> c[0]; measure q[1] -> c[1]; '
           'if (c == 2) x q[2]; if (c == 1) h q[2]; if (c == 3) y q[2];')
    p = qasm.parse(src)
    qs = _OracleStates(3)
    assert p.run(qs, randnum=[0.5, 0.5], gate_runner=_oracle_gates) == 2
    want = np.zeros(8)
    want[0b110] = 1
    assert np.allclose(qs.psi, want)
