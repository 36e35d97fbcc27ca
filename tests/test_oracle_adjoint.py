"""CPU checks of the gradient oracle and of the host-side circuit expansion
(no kernel launches)."""
import math

import numpy as np

from oracle import adjoint_oracle as ao
from oracle import statevec as sv


def _pauli_matrix(n, paulis):
    mats = {q: a for q, a in paulis}
    full = np.array([[1.]], np.complex128)
    for q in reversed(range(n)):  # lane n-1 is the most significant
        full = np.kron(full, sv.gate_matrix(mats.get(q, 'ID')) if q in mats else np.eye(2))
    return full


def test_parameter_shift_matches_finite_difference():
    from qgate_gb300.adjoint import PauliSum, ParamCircuit
    rng = np.random.default_rng(0)
    n = 4
    c = ParamCircuit(n)
    for layer in range(2):
        for q in range(n):
            c.u3(q, 3 * (layer * n + q), 3 * (layer * n + q) + 1, 3 * (layer * n + q) + 2)
        for q in range(n - 1):
            c.cx(q, q + 1)
    c.expiz(2, 3 * 2 * n)
    c.expi([(0, 'X'), (1, 'Y'), (3, 'Z')], 3 * 2 * n + 1)
    H = PauliSum.ising_chain(n).add(0.3, [(0, 'Y'), (2, 'X')])
    params = rng.uniform(-math.pi, math.pi, c.n_params)
    ps = ao.parameter_shift(n, c.ops, params, H.terms)
    fd = ao.finite_difference(n, c.ops, params, H.terms, h=1e-4)
    assert np.max(np.abs(ps - fd)) < 1e-7


def test_expi_expansion_equals_matrix_exponential():
    """Expi(theta)(P) = exp(+i theta P) through basis change + CX chain + Z
    rotation, as the reference expands it (qgate/model/expand.py:18-51)."""
    from qgate_gb300.adjoint import ParamCircuit
    n = 3
    theta = 0.37
    for paulis in ([(0, 'X')], [(1, 'Y')], [(0, 'X'), (2, 'Z')], [(0, 'Y'), (1, 'X'), (2, 'Y')]):
        c = ParamCircuit(n)
        c.expi(paulis, 0)
        U = np.zeros((8, 8), np.complex128)
        for col in range(8):
            psi = np.zeros(8, np.complex128)
            psi[col] = 1.
            for op in c.ops:
                if op[0] == 'rot':
                    _, axis, target, controls, p, coef = op
                    m = ao.rotation_matrix(axis, coef * theta)
                else:
                    kind, name, args, target, controls = op
                    m = sv.gate_matrix(name, args, adjoint=(kind == 'gate_adj'))
                sv.apply_controlled_gate(psi, m, list(controls), target)
            U[:, col] = psi
        P = _pauli_matrix(n, paulis)
        want = math.cos(theta) * np.eye(8) + 1j * math.sin(theta) * P
        assert np.allclose(U, want, atol=1e-12), paulis


def test_u3_decomposition_matches_reference_matrix():
    from qgate_gb300.adjoint import ParamCircuit
    c = ParamCircuit(1).u3(0, 0, 1, 2)
    th = [0.7, -1.2, 2.3]
    U = np.zeros((2, 2), np.complex128)
    for col in range(2):
        psi = np.zeros(2, np.complex128)
        psi[col] = 1.
        for op in c.ops:
            _, axis, target, controls, p, coef = op
            sv.apply_gate(psi, ao.rotation_matrix(axis, coef * th[p]), target)
        U[:, col] = psi
    assert np.allclose(U, sv.gate_matrix('U', tuple(th)), atol=1e-14)


def test_oracle_gradients_match_reference_parameter_shift():
    """The oracle's energy and parameter-shift gradients of the 12-qubit,
    12-layer hardware-efficient ansatz (Ry, Rz + CX ring; transverse-field
    Ising chain) equal the ones the reference computed on its own C++ CPU
    runtime in complex128 (tests/golden/gradients_hea12.npz, written by
    tests/golden/make_gradients.py)."""
    import os
    from qgate_gb300.adjoint import PauliSum, hardware_efficient_ansatz
    g = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'gradients_hea12.npz'))
    n = 12
    c = hardware_efficient_ansatz(n, 12)
    H = PauliSum.ising_chain(n)
    params = g['params']
    assert c.n_params == len(params)
    assert abs(ao.energy(n, c.ops, params, H.terms) - float(g['energy'])) < 1e-10
    ps = ao.parameter_shift(n, c.ops, params, H.terms)
    assert np.max(np.abs(ps - g['grad'])) < 1e-10
