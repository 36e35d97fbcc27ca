"""Batched execution of many small circuits of uneven qubit counts.

`sum_z(circuits)` runs every circuit from |0...0> (complex64) and returns
sum_i <Z_i> per circuit, accumulated in FP64.  The whole batch is one
persistent launch (inside a recorded CUDA graph) whose CTAs take work items
from a device-side queue: circuits of up to 12 qubits are simulated entirely
inside one CTA's shared memory / registers; larger ones advance one fused
stage at a time over a packed device arena (an item = up to eight tiles of
one stage; the queue runs round by round over all large circuits), an item
waiting until its circuit's previous stage is complete; the last items sum
each large circuit's <Z_i> (C ABI: `qg_batch_sum_z`; `qg_set_batch_one_launch`
selects the one-launch-per-round form instead).

    circuits = [(n_qubits, [(gate_name, args, target, controls), ...]), ...]
"""
import numpy as np

from . import _native as nat
from .adjoint import _COp

nat.lib.qg_batch_sum_z.argtypes = [nat._i, nat._i, nat._vp, nat._vp, nat.ctypes.POINTER(_COp),
                                   nat._vp]
nat.lib.qg_batch_sum_z.restype = nat._i


OP_DTYPE = np.dtype([('kind', '<i4'), ('target', '<i4'), ('n_controls', '<i4'),
                     ('controls', '<i4', (4,)), ('axis', '<i4'), ('param', '<i4'),
                     ('coef', '<f8'), ('mat', '<f8', (8,))], align=True)
assert OP_DTYPE.itemsize == nat.ctypes.sizeof(_COp)


def _rotation_mats(name, theta):
    """Vectorised 2x2 matrices of the one-angle rotations, in the reference's
    conventions (qgate/simulator/src/GateMatrix.cpp:114-141); rows of 8
    doubles {re00, im00, re01, im01, re10, im10, re11, im11}."""
    h = 0.5 * theta
    c, s = np.cos(h), np.sin(h)
    m = np.zeros((len(theta), 8))
    if name == 'RX':
        m[:, 0] = c; m[:, 3] = -s; m[:, 5] = -s; m[:, 6] = c
    elif name == 'RY':
        m[:, 0] = c; m[:, 2] = -s; m[:, 4] = s; m[:, 6] = c
    elif name == 'RZ':
        m[:, 0] = c; m[:, 1] = -s; m[:, 6] = c; m[:, 7] = s
    elif name == 'U1':
        m[:, 0] = 1.; m[:, 6] = np.cos(theta); m[:, 7] = np.sin(theta)
    else:
        return None
    return m


def pack(circuits):
    """(n_qubits int32[C], gate_offsets int64[C+1], gates OP_DTYPE[G])."""
    n = np.array([c[0] for c in circuits], np.int32)
    offsets = np.zeros(len(circuits) + 1, np.int64)
    offsets[1:] = np.cumsum([len(c[1]) for c in circuits])
    total = int(offsets[-1])
    gates = np.zeros(max(1, total), OP_DTYPE)
    flat = [g for _, gl in circuits for g in gl]
    if not flat:
        return n, offsets, gates
    names = np.array([g[0] for g in flat])
    gates['target'][:total] = [g[2] for g in flat]
    gates['n_controls'][:total] = [len(g[3]) for g in flat]
    gates['controls'][:total] = [tuple(g[3]) + (0,) * (4 - len(g[3])) for g in flat]
    mats = gates['mat']
    for name in np.unique(names):
        sel = np.nonzero(names == name)[0]
        args = [flat[i][1] for i in sel]
        vec = _rotation_mats(str(name), np.array([a[0] for a in args], np.float64)) \
            if len(args[0]) == 1 else None
        if vec is not None:
            mats[sel] = vec
            continue
        cache = {}
        for i, a in zip(sel, args):
            key = tuple(a)
            m = cache.get(key)
            if m is None:
                m = cache[key] = np.ascontiguousarray(
                    nat.gate_matrix(str(name), key).reshape(-1)).view(np.float64)
            mats[i] = m
    return n, offsets, gates


def sum_z(circuits=None, packed=None):
    """sum_i <Z_i> per circuit (FP64)."""
    n, offsets, gates = packed if packed is not None else pack(circuits)
    out = np.empty(len(n), np.float64)
    nat.check(nat.lib.qg_batch_sum_z(nat.PREC_FP32, len(n), n.ctypes.data, offsets.ctypes.data,
                                     gates.ctypes.data_as(nat.ctypes.POINTER(_COp)),
                                     out.ctypes.data))
    return out


def hea_batch(count=4096, seed=20, min_qubits=8, max_qubits=20, min_depth=4, max_depth=12):
    """Hardware-efficient ansatz circuits of uneven sizes: n ~ U{min..max}
    qubits, depth ~ U{min..max}; each layer is Ry and Rz on every qubit with
    angles uniform(-pi, pi), then a linear CX ladder (q_i -> q_i+1)."""
    rng = np.random.default_rng(seed)
    circuits = []
    for _ in range(count):
        n = int(rng.integers(min_qubits, max_qubits + 1))
        depth = int(rng.integers(min_depth, max_depth + 1))
        ops = []
        for _ in range(depth):
            ang = rng.uniform(-np.pi, np.pi, (n, 2))
            for q in range(n):
                ops.append(('RY', (float(ang[q, 0]),), q, ()))
                ops.append(('RZ', (float(ang[q, 1]),), q, ()))
            for q in range(n - 1):
                ops.append(('X', (), q + 1, (q,)))
        circuits.append((n, ops))
    return circuits
