"""Helpers for the GPU tests: drive the GB300 runtime through its plugin
protocol (the calls the reference front-end makes) and compare with the
oracle."""
import numpy as np

from qgate_gb300 import _native as nat
from tests.replay import make_gate_type, Lane, null, abs2  # noqa: F401

CDT = {np.float64: np.complex128, np.float32: np.complex64}
ATOL = {np.float64: 1e-12, np.float32: 2e-6}


def new_state(rt, n, dtype):
    qs = rt.create_qubit_states(dtype)
    qs.processor.initialize_qubit_states(qs, n)
    qs.processor.reset_qubit_states(qs)
    return qs


def apply_ops(qs, ops):
    """ops: ('g', name, args, adj, target, controls) tuples (oracle.statevec.run_ops format)."""
    for op in ops:
        _, name, args, adj, target, controls = op
        gt = make_gate_type(name, args)
        if controls:
            qs.processor.apply_controlled_gate(gt, adj, qs, list(controls), target)
        else:
            qs.processor.apply_gate(gt, adj, qs, target)


GATES1 = [('H', ()), ('X', ()), ('Y', ()), ('Z', ()), ('S', ()), ('T', ()), ('SH', ()),
          ('RX', (0.7,)), ('RY', (-1.3,)), ('RZ', (2.1,)), ('U1', (0.4,)), ('U2', (0.3, -0.8)),
          ('ExpiI', (0.25,)), ('ExpiZ', (-0.6,))]


def random_ops(rng, n, count, max_controls=2, p_ctrl=0.35):
    ops = []
    for _ in range(count):
        if rng.random() < 0.45:
            name, args = 'U', tuple(rng.uniform(0, 2 * np.pi, 3))
        else:
            name, args = GATES1[rng.integers(len(GATES1))]
        lanes = rng.permutation(n)
        target = int(lanes[0])
        nc = 0
        if n > 1 and rng.random() < p_ctrl:
            nc = int(rng.integers(1, min(max_controls, n - 1) + 1))
        ctrls = tuple(int(x) for x in lanes[1:1 + nc])
        ops.append(('g', name, args, bool(rng.random() < 0.2), target, ctrls))
    return ops


def fidelity_error(a, b):
    a = a.astype(np.complex128)
    b = b.astype(np.complex128)
    return abs(1. - abs(np.vdot(a, b)))
