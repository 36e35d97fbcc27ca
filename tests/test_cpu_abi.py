"""CPU-only checks of the C ABI: the library loads, exports every entry point
declared in include/qgate_gb300.h, and its host-side gate-matrix factory
matches the reference's matrices.  No kernel is launched here."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, 'include', 'qgate_gb300.h')
GOLDEN = os.path.join(ROOT, 'tests', 'golden', 'gate_matrices.npz')


def header_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r'^\s*(?:int|const char \*)\s*(qg_\w+)\s*\(', text, re.M)))


def test_header_declares_entry_points():
    syms = header_symbols()
    assert 'qg_qubit_processor_apply_gate' in syms
    assert len(syms) >= 30


def test_library_exports_every_declared_symbol():
    from qgate_gb300 import _native
    missing = [s for s in header_symbols() if not hasattr(_native.lib, s)]
    assert not missing, missing


def test_ctypes_signatures_cover_header():
    from qgate_gb300 import _native
    syms = set(header_symbols()) - {'qg_last_error'}
    assert syms == set(_native.SIGNATURES), syms ^ set(_native.SIGNATURES)


def _golden_matrices():
    d = np.load(GOLDEN)
    for key, mat in zip(d['keys'], d['mats']):
        name, args, _ = str(key).split('|')
        args = tuple(float(a) for a in args.split(',')) if args else ()
        yield name, args, mat


def test_abi_gate_matrices_match_reference():
    from qgate_gb300 import _native
    n = 0
    for name, args, mat in _golden_matrices():
        got = _native.gate_matrix(name, args)
        assert np.allclose(got, mat, atol=1e-15, rtol=0), (name, args)
        adj = _native.gate_matrix(name, args, adjoint=True)
        assert np.allclose(adj, mat.conj().T, atol=1e-15, rtol=0), (name, args)
        n += 1
    assert n > 100


def test_oracle_gate_matrices_match_reference():
    from oracle import statevec as sv
    for name, args, mat in _golden_matrices():
        assert np.allclose(sv.gate_matrix(name, args), mat, atol=1e-15, rtol=0), (name, args)


def test_unknown_gate_raises():
    from qgate_gb300 import _native
    with pytest.raises(RuntimeError, match='Unknown gate type'):
        _native.gate_matrix('FOO')
    with pytest.raises(ValueError):
        _native.gate_matrix('U', (1.0,))


def test_invalid_handles_are_rejected_without_gpu():
    from qgate_gb300 import _native as nat
    with pytest.raises(ValueError):
        nat.call('qg_qubit_states_delete', 12345)
    with pytest.raises(ValueError):
        nat.new_handle('qg_qubit_states_new', 7)


def test_known_answer_u_gate_equals_paulis_up_to_phase():
    # qgate's U3/U2/U1 against X/Y/Z/H up to the global phase i
    # (the relations the reference checks in tests/test_U_gate.py).
    from qgate_gb300 import _native as nat
    pi = np.pi
    assert np.allclose(nat.gate_matrix('U', (pi, 0., pi)), -1j * nat.gate_matrix('X'))
    assert np.allclose(nat.gate_matrix('U', (pi, pi / 2., pi / 2.)), -1j * nat.gate_matrix('Y'))
    assert np.allclose(nat.gate_matrix('U1', (pi,)), nat.gate_matrix('Z'))
    assert np.allclose(nat.gate_matrix('U2', (0., pi)), -1j * nat.gate_matrix('H'))


def test_compiled_circuit_table_validation():
    """qg_circuit_new checks the gate table as apply_controlled_gate checks a
    call (lane range, control/target overlap, offsets) without touching the
    device; a circuit that never ran is deleted without it too."""
    from qgate_gb300 import _native as nat
    from qgate_gb300.circuit import gate_type
    from qgate_gb300.compiled import CompiledCircuit
    h, x = gate_type('H'), gate_type('X')
    c = CompiledCircuit(np.float64, [(h, False, 0, []), (x, False, 3, [0, 1]), (h, True, 61, [])],
                        graph=False)
    assert c.n_gates == 3
    c.delete()
    with pytest.raises(RuntimeError, match='overlapped'):
        CompiledCircuit(np.float32, [(x, False, 2, [1, 2])], graph=False)
    with pytest.raises(ValueError, match='out of range'):
        CompiledCircuit(np.float32, [(h, False, 62, [])], graph=False)
    with pytest.raises(ValueError, match='out of range'):
        CompiledCircuit(np.float32, [(x, False, 1, [-1])], graph=False)
    bad = nat.int_array([0, 1, 0])  # offsets must not decrease
    t = nat.int_array([0, 1])
    m = np.zeros(16)
    with pytest.raises(ValueError, match='offsets'):
        nat.new_handle('qg_circuit_new', nat.PREC_FP32, 2, nat.as_iptr(t), nat.as_iptr(bad),
                       nat.as_iptr(nat.int_array([2])), nat.as_dptr(m))
    with pytest.raises(ValueError, match='invalid circuit'):
        nat.call('qg_circuit_run', 12345, 0)
