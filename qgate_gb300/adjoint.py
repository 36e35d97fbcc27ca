"""Adjoint differentiation of Pauli-sum expectations on the GB300 engine.

A parametrised circuit is a list of fixed gates and Pauli rotations
exp(-i c theta G).  `expectation_and_gradient` evaluates E_b = <psi_b|H|psi_b>
for a batch of parameter vectors in one call and, by the adjoint method, the
gradient dE_b/dtheta (one forward sweep, one reverse sweep that un-applies the
gates from psi and lambda = H psi); `expectation` wraps it as a
`torch.autograd.Function`.

Gate conventions are the reference's (qgate/simulator/src/GateMatrix.cpp):
Rx/Ry/Rz(theta) = exp(-i theta/2 {X,Y,Z}); U(theta, phi, lambda) =
Rz(phi) Ry(theta) Rz(lambda) exactly; ExpiZ(theta) = exp(+i theta Z);
Expi(theta)(P) = exp(+i theta P), expanded like the reference's
PauliGatesDiagonalizer (qgate/model/pauli_gates_diagonalizer.py:96-135):
basis change to Z, a CX parity chain onto one lane, the Z rotation, undo.
"""
import ctypes

import numpy as np

from . import _native as nat


class _COp(ctypes.Structure):
    _fields_ = [('kind', ctypes.c_int), ('target', ctypes.c_int), ('n_controls', ctypes.c_int),
                ('controls', ctypes.c_int * 4), ('axis', ctypes.c_int), ('param', ctypes.c_int),
                ('coef', ctypes.c_double), ('mat', ctypes.c_double * 8)]


class _CTerm(ctypes.Structure):
    _fields_ = [('coef', ctypes.c_double), ('x_mask', ctypes.c_uint64),
                ('z_mask', ctypes.c_uint64)]


nat.lib.qg_adjoint_expectation.argtypes = [
    ctypes.c_int, ctypes.c_int, ctypes.POINTER(_COp), ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
    ctypes.c_int, ctypes.POINTER(_CTerm), ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
    ctypes.c_void_p]
nat.lib.qg_adjoint_expectation.restype = ctypes.c_int

AXES = {'X': 1, 'Y': 2, 'Z': 3}


class ParamCircuit:
    """Builder of a parametrised circuit on `n_qubits` lanes.

    Ops are tuples ('rot', axis, target, controls, param, coef) or
    ('gate', name, args, target, controls)."""

    def __init__(self, n_qubits):
        self.n_qubits = n_qubits
        self.ops = []
        self.n_params = 0

    def _p(self, p):
        self.n_params = max(self.n_params, p + 1)
        return p

    def gate(self, name, target, controls=(), args=()):
        self.ops.append(('gate', name, tuple(args), target, tuple(controls)))
        return self

    def cx(self, control, target):
        return self.gate('X', target, (control,))

    def rot(self, axis, target, param, coef, controls=()):
        self.ops.append(('rot', AXES[axis], target, tuple(controls), self._p(param), coef))
        return self

    def rx(self, target, param, controls=()):
        return self.rot('X', target, param, 0.5, controls)

    def ry(self, target, param, controls=()):
        return self.rot('Y', target, param, 0.5, controls)

    def rz(self, target, param, controls=()):
        return self.rot('Z', target, param, 0.5, controls)

    def u3(self, target, p_theta, p_phi, p_lambda):
        """qgate's U(theta, phi, lambda) = Rz(phi) Ry(theta) Rz(lambda)."""
        return self.rz(target, p_lambda).ry(target, p_theta).rz(target, p_phi)

    def expiz(self, target, param):
        """ExpiZ(theta) = exp(+i theta Z)."""
        return self.rot('Z', target, param, -1.0)

    def expi(self, paulis, param):
        """Expi(theta)(P) = exp(+i theta P) for a Pauli string given as
        [(qubit, 'X'|'Y'|'Z'), ...]."""
        paulis = [(q, a) for q, a in paulis if a != 'I']
        if not paulis:
            raise ValueError('empty Pauli string')
        pre = []
        for q, a in paulis:
            if a == 'X':
                pre.append(('gate', 'H', (), q, ()))
            elif a == 'Y':  # H S^dagger maps Y to Z
                pre.append(('gate_adj', 'S', (), q, ()))
                pre.append(('gate', 'H', (), q, ()))
        lanes = [q for q, _ in paulis]
        pivot = lanes[-1]
        chain = [('gate', 'X', (), lanes[i + 1], (lanes[i],)) for i in range(len(lanes) - 1)]
        body = pre + chain
        for op in body:
            self._append_fixed(op, adjoint=False)
        self.rot('Z', pivot, param, -1.0)
        for op in reversed(body):
            self._append_fixed(op, adjoint=True)
        return self

    def _append_fixed(self, op, adjoint):
        kind, name, args, target, controls = op
        adj = (kind == 'gate_adj') != adjoint
        self.ops.append(('gate_adj' if adj else 'gate', name, args, target, controls))

    def _cops(self):
        arr = (_COp * max(1, len(self.ops)))()
        for i, op in enumerate(self.ops):
            c = arr[i]
            if op[0] == 'rot':
                _, axis, target, controls, param, coef = op
                c.kind, c.axis, c.param, c.coef = 1, axis, param, coef
            else:
                kind, name, args, target, controls = op
                m = nat.gate_matrix(name, args, adjoint=(kind == 'gate_adj'))
                c.kind = 0
                flat = np.ascontiguousarray(m.reshape(-1)).view(np.float64)
                for k in range(8):
                    c.mat[k] = flat[k]
            c.target = target
            c.n_controls = len(controls)
            for k, q in enumerate(controls):
                c.controls[k] = q
        return arr


class PauliSum:
    """Observable sum_t coef_t P_t; P_t given by (x_mask, z_mask)."""

    def __init__(self, terms=()):
        self.terms = list(terms)

    def add(self, coef, paulis):
        x = z = 0
        for q, a in paulis:
            if a in ('X', 'Y'):
                x |= 1 << q
            if a in ('Z', 'Y'):
                z |= 1 << q
        self.terms.append((float(coef), x, z))
        return self

    @staticmethod
    def ising_chain(n, J=1.0, h=0.7):
        """H = -J sum_{i<n-1} Z_i Z_{i+1} - h sum_i X_i (open chain)."""
        H = PauliSum()
        for i in range(n - 1):
            H.add(-J, [(i, 'Z'), (i + 1, 'Z')])
        for i in range(n):
            H.add(-h, [(i, 'X')])
        return H

    def _cterms(self):
        arr = (_CTerm * len(self.terms))()
        for i, (c, x, z) in enumerate(self.terms):
            arr[i].coef, arr[i].x_mask, arr[i].z_mask = c, x, z
        return arr


def expectation_and_gradient(circuit, params, observable, dtype=np.float32, checkpoint_every=0,
                             gradient=True):
    """E (batch,) and dE/dparams (batch, n_params) for params of shape
    (batch, n_params) (or (n_params,)).  dtype: np.float32 (complex64
    states) or np.float64 (complex128); accumulation is FP64 either way."""
    p = np.ascontiguousarray(np.atleast_2d(np.asarray(params, np.float64)))
    batch, n_params = p.shape
    if n_params < circuit.n_params:
        raise ValueError('circuit uses %d parameters, got %d' % (circuit.n_params, n_params))
    E = np.empty(batch, np.float64)
    G = np.empty((batch, n_params), np.float64) if gradient else None
    prec = nat.PREC_FP64 if dtype == np.float64 else nat.PREC_FP32
    ops = circuit._cops()
    terms = observable._cterms()
    nat.check(nat.lib.qg_adjoint_expectation(
        prec, circuit.n_qubits, ops, len(circuit.ops), p.ctypes.data, n_params, batch, terms,
        len(observable.terms), int(checkpoint_every), E.ctypes.data,
        G.ctypes.data if gradient else None))
    return E, G


def _torch_function():
    import torch

    class AdjointExpectation(torch.autograd.Function):
        """E = <psi(theta)|H|psi(theta)> with the adjoint-method backward."""

        @staticmethod
        def forward(ctx, params, circuit, observable, dtype, checkpoint_every):
            p = params.detach().to('cpu', torch.float64).numpy()
            E, G = expectation_and_gradient(circuit, p, observable, dtype, checkpoint_every,
                                            gradient=params.requires_grad)
            if G is not None:
                ctx.save_for_backward(torch.from_numpy(G).to(params.device, params.dtype))
            out = torch.from_numpy(E).to(params.device, params.dtype)
            return out if params.dim() == 2 else out[0]

        @staticmethod
        def backward(ctx, grad_out):
            (G,) = ctx.saved_tensors
            g = grad_out.reshape(-1, 1) * G
            if grad_out.dim() == 0:
                g = g[0]
            return g, None, None, None, None

    return AdjointExpectation


_fn = None


def expectation(params, circuit, observable, dtype=np.float32, checkpoint_every=0):
    """torch entry point: `params` (n_params,) or (batch, n_params) tensor;
    returns E with an autograd backward computed by the adjoint method."""
    global _fn
    if _fn is None:
        _fn = _torch_function()
    return _fn.apply(params, circuit, observable, dtype, checkpoint_every)


def hardware_efficient_ansatz(n, layers, ring=True):
    """Layers of Ry and Rz on every qubit followed by a CX ring (or ladder);
    parameters numbered layer-major (2 n per layer)."""
    c = ParamCircuit(n)
    p = 0
    for _ in range(layers):
        for q in range(n):
            c.ry(q, p)
            p += 1
        for q in range(n):
            c.rz(q, p)
            p += 1
        for q in range(n - 1 if not ring else n):
            c.cx(q, (q + 1) % n)
    return c
