"""GPU parity of the adjoint-gradient engine.

Expectations against the oracle's complex128 run; gradients against the
oracle's parameter-shift (uncontrolled rotations) or central finite
differences (controlled rotations), i.e. the gradients a user of the
reference obtains by re-running its simulation with shifted parameters.
Tolerances: complex128 1e-10; complex64 1e-5 (the target bound for FP32
gradients)."""
import math

import numpy as np
import pytest

from oracle import adjoint_oracle as ao

pytestmark = pytest.mark.gpu

DTYPES = [np.float64, np.float32]
IDS = ['c128', 'c64']
TOL = {np.float64: 1e-10, np.float32: 1e-5}


def _random_circuit(rng, n, layers, controlled=False):
    from qgate_gb300.adjoint import ParamCircuit
    c = ParamCircuit(n)
    p = 0
    for _ in range(layers):
        for q in range(n):
            c.u3(q, p, p + 1, p + 2)
            p += 3
        for q in range(n - 1):
            c.cx(q, q + 1)
        c.gate('H', int(rng.integers(n)))
        c.rx(int(rng.integers(n)), p)
        p += 1
        c.expiz(int(rng.integers(n)), p)
        p += 1
        a, b = rng.permutation(n)[:2]
        c.expi([(int(a), 'X'), (int(b), 'Y')], p)
        p += 1
        if controlled:
            a, b = rng.permutation(n)[:2]
            c.ry(int(b), p, controls=(int(a),))
            p += 1
    return c


def _observable(rng, n):
    from qgate_gb300.adjoint import PauliSum
    H = PauliSum.ising_chain(n, 1.0, 0.7)
    for _ in range(4):
        qs = rng.permutation(n)[:3]
        H.add(float(rng.normal()), [(int(qs[0]), 'X'), (int(qs[1]), 'Y'), (int(qs[2]), 'Z')])
    return H


@pytest.mark.parametrize('n', [3, 9, 13])
@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_adjoint_matches_parameter_shift(n, dtype):
    from qgate_gb300.adjoint import expectation_and_gradient
    rng = np.random.default_rng(n)
    c = _random_circuit(rng, n, 2)
    H = _observable(rng, n)
    params = rng.uniform(-math.pi, math.pi, (2, c.n_params))
    E, G = expectation_and_gradient(c, params, H, dtype)
    for b in range(2):
        e_ref = ao.energy(n, c.ops, params[b], H.terms)
        g_ref = ao.parameter_shift(n, c.ops, params[b], H.terms)
        assert abs(E[b] - e_ref) < TOL[dtype], (E[b], e_ref)
        assert np.max(np.abs(G[b] - g_ref)) < TOL[dtype], np.max(np.abs(G[b] - g_ref))


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_adjoint_controlled_rotations_vs_finite_difference(dtype):
    from qgate_gb300.adjoint import expectation_and_gradient
    rng = np.random.default_rng(5)
    n = 10
    c = _random_circuit(rng, n, 2, controlled=True)
    H = _observable(rng, n)
    params = rng.uniform(-math.pi, math.pi, c.n_params)
    E, G = expectation_and_gradient(c, params, H, dtype)
    fd = ao.finite_difference(n, c.ops, params, H.terms, h=1e-4)
    assert np.max(np.abs(G[0] - fd)) < max(TOL[dtype], 1e-7)


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_checkpoints_and_batch_consistency(dtype):
    """Re-anchoring at checkpoints gives the same answer; a batch equals the
    individual evaluations."""
    from qgate_gb300.adjoint import expectation_and_gradient, hardware_efficient_ansatz, PauliSum
    n = 12
    c = hardware_efficient_ansatz(n, 6)
    H = PauliSum.ising_chain(n)
    rng = np.random.default_rng(9)
    params = rng.uniform(-math.pi, math.pi, (3, c.n_params))
    E0, G0 = expectation_and_gradient(c, params, H, dtype)
    E1, G1 = expectation_and_gradient(c, params, H, dtype, checkpoint_every=3 * (2 * n + n))
    assert np.max(np.abs(E0 - E1)) < TOL[dtype]
    assert np.max(np.abs(G0 - G1)) < TOL[dtype]
    for b in range(3):
        e, g = expectation_and_gradient(c, params[b], H, dtype)
        assert abs(e[0] - E0[b]) < 1e-12 * max(1, abs(e[0])) + TOL[dtype] * 1e-2
        assert np.max(np.abs(g[0] - G0[b])) < TOL[dtype]
    g_ref = ao.parameter_shift(n, c.ops, params[1], H.terms)
    assert np.max(np.abs(G1[1] - g_ref)) < TOL[dtype]


def test_fp32_gradients_track_fp64_at_24_qubits():
    """The benchmark's ansatz (24 qubits, 12 layers of Ry, Rz + CX ring, 576
    parameters, transverse-field Ising chain): complex64 gradients with
    checkpoints vs the engine's complex128 gradients, and a seeded subset of
    complex128 gradients vs central finite differences of the complex128
    energy (h = 1e-3)."""
    from qgate_gb300.adjoint import expectation_and_gradient, hardware_efficient_ansatz, PauliSum
    n = 24
    c = hardware_efficient_ansatz(n, 12)
    H = PauliSum.ising_chain(n)
    params = np.random.default_rng(30).uniform(-math.pi, math.pi, (2, c.n_params))
    E64, G64 = expectation_and_gradient(c, params, H, np.float64)
    E32, G32 = expectation_and_gradient(c, params, H, np.float32, checkpoint_every=3 * 72)
    assert np.max(np.abs(E32 - E64)) < 1e-5
    assert np.max(np.abs(G32 - G64)) < 1e-5, np.max(np.abs(G32 - G64))
    rng = np.random.default_rng(31)
    h = 1e-3
    for k in rng.choice(c.n_params, 6, replace=False):
        pp = np.repeat(params[:1], 2, axis=0)
        pp[0, k] += h
        pp[1, k] -= h
        E, _ = expectation_and_gradient(c, pp, H, np.float64, gradient=False)
        fd = (E[0] - E[1]) / (2 * h)
        assert abs(fd - G64[0, k]) < 1e-5, (k, fd, G64[0, k])


def test_torch_autograd_function():
    import torch
    from qgate_gb300.adjoint import expectation, hardware_efficient_ansatz, PauliSum
    n = 8
    c = hardware_efficient_ansatz(n, 3)
    H = PauliSum.ising_chain(n)
    theta = torch.tensor(np.random.default_rng(2).uniform(-3, 3, c.n_params),
                         dtype=torch.float64, requires_grad=True)
    E = expectation(theta, c, H, np.float64)
    E.backward()
    g_ref = ao.parameter_shift(n, c.ops, theta.detach().numpy(), H.terms)
    assert abs(E.item() - ao.energy(n, c.ops, theta.detach().numpy(), H.terms)) < 1e-10
    assert np.max(np.abs(theta.grad.numpy() - g_ref)) < 1e-10
    # batched: sum of energies
    thetas = torch.tensor(np.random.default_rng(3).uniform(-3, 3, (4, c.n_params)),
                          dtype=torch.float64, requires_grad=True)
    Eb = expectation(thetas, c, H, np.float64)
    Eb.sum().backward()
    for b in range(4):
        g = ao.parameter_shift(n, c.ops, thetas.detach().numpy()[b], H.terms)
        assert np.max(np.abs(thetas.grad.numpy()[b] - g)) < 1e-10


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_adjoint_matches_reference_parameter_shift(dtype):
    """The engine's adjoint gradients of the 12-qubit, 12-layer
    hardware-efficient ansatz (288 parameters) against the parameter-shift
    gradients the reference computed on its own C++ CPU runtime in complex128
    (tests/golden/gradients_hea12.npz).  complex128 1e-10, complex64 1e-5."""
    import os
    from qgate_gb300.adjoint import expectation_and_gradient, hardware_efficient_ansatz, PauliSum
    g = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'gradients_hea12.npz'))
    n = 12
    c = hardware_efficient_ansatz(n, 12)
    H = PauliSum.ising_chain(n)
    E, G = expectation_and_gradient(c, g['params'], H, dtype, checkpoint_every=3 * 3 * n)
    assert abs(E[0] - float(g['energy'])) < TOL[dtype]
    assert np.max(np.abs(G[0] - g['grad'])) < TOL[dtype], np.max(np.abs(G[0] - g['grad']))
