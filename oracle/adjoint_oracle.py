"""CPU oracle for expectations and gradients of parametrised circuits.

TEST INFRASTRUCTURE ONLY (part of the oracle; never called by the product).

The reference has no gradient path: its users differentiate by running the
circuit again with shifted parameters (parameter-shift) or by finite
differences, each run being the reference's ordinary simulation
(qgate/simulator/simulator.py:57-83).  This module does exactly that on the
oracle's complex128 state vector (oracle.statevec, pinned to the
reference's own runtime): `parameter_shift` for circuits whose parametrised
gates are uncontrolled Pauli rotations exp(-i c theta G) (G^2 = I, so
dE/dtheta = c [E(theta + pi/(4c)) - E(theta - pi/(4c))] per occurrence:
Rx/Ry/Rz shift pi/2 with factor 1/2, ExpiZ shift pi/4 with factor 1), and
`finite_difference` (central) for anything else.

Ops use the parametrised-circuit tuple format: ('rot', axis(1=X,2=Y,3=Z),
target, controls, param, coef) and ('gate'|'gate_adj', name, args, target,
controls).
"""
import math

import numpy as np

from . import statevec as sv

_PAULI = {1: 'X', 2: 'Y', 3: 'Z'}


def rotation_matrix(axis, angle):
    """exp(-i angle G) = cos(angle) I - i sin(angle) G."""
    g = sv.gate_matrix(_PAULI[axis])
    return math.cos(angle) * np.eye(2, dtype=np.complex128) - 1j * math.sin(angle) * g


def run(n, ops, params):
    psi = sv.initial_state(n)
    for op in ops:
        if op[0] == 'rot':
            _, axis, target, controls, p, coef = op
            m = rotation_matrix(axis, coef * params[p])
        else:
            kind, name, args, target, controls = op
            m = sv.gate_matrix(name, args, adjoint=(kind == 'gate_adj'))
        sv.apply_controlled_gate(psi, m, list(controls), target)
    return psi


def expectation(psi, terms):
    return sum(c * sv.pauli_expectation(psi, x, z) for c, x, z in terms)


def energy(n, ops, params, terms):
    return expectation(run(n, ops, params), terms)


def parameter_shift(n, ops, params, terms):
    params = np.asarray(params, np.float64)
    grad = np.zeros_like(params)
    for k, op in enumerate(ops):
        if op[0] != 'rot':
            continue
        _, axis, target, controls, p, coef = op
        if controls:
            raise ValueError('parameter-shift needs uncontrolled rotations')
        shift = math.pi / (4. * coef)
        for sign in (1., -1.):
            shifted = list(ops)
            # shift this occurrence only: a private parameter slot
            shifted[k] = ('rot', axis, target, controls, len(params), coef)
            pe = np.append(params, params[p] + sign * shift)
            grad[p] += sign * coef * energy(n, shifted, pe, terms)
    return grad


def finite_difference(n, ops, params, terms, h=1e-3, indices=None):
    params = np.asarray(params, np.float64)
    idx = range(len(params)) if indices is None else indices
    grad = np.zeros(len(params))
    for p in idx:
        e = np.zeros_like(params)
        e[p] = h
        grad[p] = (energy(n, ops, params + e, terms) - energy(n, ops, params - e, terms)) / (2 * h)
    return grad
