"""CPU oracle: a numpy restatement of the reference's state-vector primitives.

TEST INFRASTRUCTURE ONLY.  This module is the oracle for the GB300 engine:
only `tests/`, `__graft_entry__.smoke()` and the `cpu_baseline` leg of
`bench.py` may import it.  The product (`qgate_gb300`) never calls it and has
no CPU fallback.

Every function restates the algorithm of the reference file:line it names
(qgate 0.2.2).  States are complex128 (the reference's FP64 oracle runtime)
unless a complex64 array is passed in.  Index bit i of an amplitude is local
lane i.  The restatement is pinned against golden vectors produced by running
the reference itself (`tests/golden/make_golden.py`, replayed by
`tests/test_oracle_replay.py`), the matrices recorded from it
(`tests/test_cpu_abi.py`) and its parameter-shift gradients
(`tests/test_oracle_adjoint.py`).
"""
import cmath
import math

import numpy as np


# ------------------------------------------------------------------ gate matrices

def gate_matrix(name, args=(), adjoint=False):
    """2x2 matrix of a named gate: qgate/simulator/src/GateMatrix.cpp:13-158,
    qgate/simulator/pymatrix.py:18-149.  U(theta, phi, lambda) is
    Rz(phi) Ry(theta) Rz(lambda) (OpenQASM's U up to exp(i(lambda+phi)/2))."""
    j = 1j
    r = math.sqrt(0.5)
    if name == 'U':
        t, p, l = args
        c, s = math.cos(t / 2.), math.sin(t / 2.)
        m = [[cmath.exp(0.5j * (-l - p)) * c, -cmath.exp(0.5j * (l - p)) * s],
             [cmath.exp(0.5j * (-l + p)) * s, cmath.exp(0.5j * (l + p)) * c]]
    elif name == 'U2':
        p, l = args
        m = [[cmath.exp(0.5j * (-l - p)) * r, -cmath.exp(0.5j * (l - p)) * r],
             [cmath.exp(0.5j * (-l + p)) * r, cmath.exp(0.5j * (l + p)) * r]]
    elif name == 'U1':
        l, = args
        m = [[1., 0.], [0., cmath.exp(j * l)]]
    elif name == 'ID':
        m = [[1., 0.], [0., 1.]]
    elif name == 'X':
        m = [[0., 1.], [1., 0.]]
    elif name == 'Y':
        m = [[0., -j], [j, 0.]]
    elif name == 'Z':
        m = [[1., 0.], [0., -1.]]
    elif name == 'H':
        m = [[r, r], [r, -r]]
    elif name == 'S':
        m = [[1., 0.], [0., j]]
    elif name == 'T':
        m = [[1., 0.], [0., cmath.exp(j * math.pi / 4.)]]
    elif name == 'RX':
        t, = args
        c, s = math.cos(t / 2.), math.sin(t / 2.)
        m = [[c, -j * s], [-j * s, c]]
    elif name == 'RY':
        t, = args
        c, s = math.cos(t / 2.), math.sin(t / 2.)
        m = [[c, -s], [s, c]]
    elif name == 'RZ':
        t, = args
        m = [[cmath.exp(-j * t / 2.), 0.], [0., cmath.exp(j * t / 2.)]]
    elif name == 'ExpiI':
        t, = args
        m = [[cmath.exp(j * t), 0.], [0., cmath.exp(j * t)]]
    elif name == 'ExpiZ':
        t, = args
        m = [[cmath.exp(j * t), 0.], [0., cmath.exp(-j * t)]]
    elif name == 'SH':
        m = [[r, r], [j * r, -j * r]]
    else:
        raise RuntimeError('Unknown gate type.')
    m = np.array(m, np.complex128)
    if adjoint:  # qgate/simulator/src/GateMatrix.cpp:150-158
        m = m.conj().T.copy()
    return m


# ------------------------------------------------------------------ state helpers

def _split(psi, lane):
    """View of psi as [hi, 2, lo] with the middle axis = lane bit."""
    n = psi.size
    lo = 1 << lane
    return psi.reshape(n // (2 * lo), 2, lo)


def initial_state(n, dtype=np.complex128):
    """|0...0>: qgate/simulator/src/CPUQubitProcessor.cpp:61-73."""
    psi = np.zeros(1 << n, dtype)
    psi[0] = 1.
    return psi


def apply_gate(psi, mat, lane):
    """(psi[i0], psi[i1]) <- mat (psi[i0], psi[i1]) for all pairs that differ
    in `lane`: qgate/simulator/src/CPUQubitProcessor.cpp:307-329,
    qgate/simulator/pyruntime.py:149-167."""
    v = _split(psi, lane)
    m = mat.astype(psi.dtype)
    a, b = v[:, 0, :].copy(), v[:, 1, :].copy()
    v[:, 0, :] = m[0, 0] * a + m[0, 1] * b
    v[:, 1, :] = m[1, 0] * a + m[1, 1] * b
    return psi


def apply_controlled_gate(psi, mat, controls, target):
    """The same 2x2 update restricted to indices whose control bits are all 1:
    qgate/simulator/src/CPUQubitProcessor.cpp:331-362,
    qgate/simulator/pyruntime.py:169-210."""
    if not controls:
        return apply_gate(psi, mat, target)
    n = int(psi.size).bit_length() - 1
    idx = np.arange(psi.size, dtype=np.int64)
    cmask = 0
    for c in controls:
        cmask |= 1 << c
    tbit = 1 << target
    sel = idx[((idx & cmask) == cmask) & ((idx & tbit) == 0)]
    m = mat.astype(psi.dtype)
    a, b = psi[sel].copy(), psi[sel | tbit].copy()
    psi[sel] = m[0, 0] * a + m[0, 1] * b
    psi[sel | tbit] = m[1, 0] * a + m[1, 1] * b
    del n
    return psi


def apply_matrix(psi, mat, targets, controls=()):
    """Dense 2^k x 2^k matrix on `targets` (targets[0] = matrix bit 0), the
    composition the reference expresses as sequences of 1-qubit and
    controlled gates (e.g. SWAP = 3 CX, qgate/model/expand.py:14-16)."""
    k = len(targets)
    idx = np.arange(psi.size, dtype=np.int64)
    tmask = 0
    for t in targets:
        tmask |= 1 << t
    cmask = 0
    for c in controls:
        cmask |= 1 << c
    base = idx[((idx & tmask) == 0) & ((idx & cmask) == cmask)]
    offs = np.zeros(1 << k, np.int64)
    for jj in range(1 << k):
        o = 0
        for b, t in enumerate(targets):
            if jj & (1 << b):
                o |= 1 << t
        offs[jj] = o
    gidx = base[:, None] | offs[None, :]
    vals = psi[gidx]
    psi[gidx] = vals @ mat.astype(psi.dtype).T
    return psi


def calc_probability(psi, lane):
    """Pr(lane == 0) = sum over indices with the lane bit clear of |psi|^2:
    qgate/simulator/src/CPUQubitProcessor.cpp:75-125,
    qgate/simulator/pyruntime.py:55-67."""
    v = _split(psi, lane)[:, 0, :]
    return float(np.sum(v.real.astype(np.float64) ** 2 + v.imag.astype(np.float64) ** 2))


def decohere(psi, value, prob, lane):
    """Collapse of a measured lane: qgate/simulator/src/CPUQubitProcessor.cpp:217-246,
    qgate/simulator/pyruntime.py:84-106."""
    v = _split(psi, lane)
    if value == 0:
        v[:, 0, :] *= 1. / math.sqrt(prob)
        v[:, 1, :] = 0.
    else:
        v[:, 0, :] = 0.
        v[:, 1, :] *= 1. / math.sqrt(1. - prob)
    return psi


def decohere_and_separate(psi, value, prob, lane):
    """Returns (psi0 on n-1 lanes, psi1 = |value>):
    qgate/simulator/src/CPUQubitProcessor.cpp:248-284,
    qgate/simulator/pyruntime.py:108-133."""
    v = _split(psi, lane)
    if value == 0:
        psi0 = (v[:, 0, :] * (1. / math.sqrt(prob))).reshape(-1)
        psi1 = np.array([1., 0.], psi.dtype)
    else:
        psi0 = (v[:, 1, :] * (1. / math.sqrt(1. - prob))).reshape(-1)
        psi1 = np.array([0., 1.], psi.dtype)
    return psi0.astype(psi.dtype), psi1


def apply_reset(psi, lane):
    """psi[i0] <- psi[i1], psi[i1] <- 0: qgate/simulator/src/CPUQubitProcessor.cpp:286-305,
    qgate/simulator/pyruntime.py:135-147."""
    v = _split(psi, lane)
    v[:, 0, :] = v[:, 1, :]
    v[:, 1, :] = 0.
    return psi


def join(states, n_new_lanes):
    """Kronecker product of the listed states (the last one in the lowest
    lanes) followed by zero-filled new |0> lanes above them:
    qgate/simulator/pyruntime.py:69-82, qgate/simulator/src/CPUQubitProcessor.cpp:129-213."""
    vec = states[0]
    for s in states[1:]:
        vec = np.kron(vec, s)
    out = np.zeros(vec.size << n_new_lanes, vec.dtype)
    out[:vec.size] = vec
    return out


# ------------------------------------------------------------------ getter / pool

def get_states(lane_trans, mathop, n_states, start, step, empty_lane_mask=0, dtype=None):
    """value[i] = prod_g op(psi_g[local_g(start + step*i)]), 0 where an empty
    lane bit is set: qgate/simulator/pyruntime.py:215-245,
    qgate/simulator/src/CPUQubitsStatesGetter.cpp:34-157.

    lane_trans: [(psi_g, [external lane of local lane l for l in lanes])].
    mathop: 'null' (amplitudes) or 'abs2' (probabilities)."""
    ext = start + step * np.arange(n_states, dtype=np.int64)
    if mathop == 'null':
        dtype = dtype or lane_trans[0][0].dtype
        val = np.ones(n_states, dtype)
    else:
        dtype = dtype or (np.float64 if lane_trans[0][0].dtype == np.complex128 else np.float32)
        val = np.ones(n_states, dtype)
    for psi, table in lane_trans:
        local = np.zeros(n_states, np.int64)
        for l, e in enumerate(table):
            local |= ((ext >> e) & 1) << l
        s = psi[local]
        val *= s if mathop == 'null' else (s.real ** 2 + s.imag ** 2).astype(dtype)
    val[(ext & empty_lane_mask) != 0] = 0.
    return val


def marginal_probabilities(lane_trans, n_lanes, n_hidden):
    """Probabilities over the 2^n_lanes pool lanes with the hidden lanes
    (external lanes n_lanes..n_lanes+n_hidden-1, i.e. placed in the MSBs as in
    qgate/simulator/cudaruntime.py:64-72) summed out:
    qgate/simulator/src/CPUQubitsStatesGetter.cpp:159-254,
    qgate/simulator/pyruntime.py:247-276.  FP64."""
    lt = [(psi.astype(np.complex128), table) for psi, table in lane_trans]
    full = get_states(lt, 'abs2', 1 << (n_lanes + n_hidden), 0, 1)
    return full.reshape(1 << n_hidden, 1 << n_lanes).sum(axis=0)


def insert_zero_bits(values, positions):
    """Insert a zero bit at each (ascending) position: the empty-lane shift of
    qgate/simulator/pyruntime.py:303-321 / BitPermTable
    (qgate/simulator/src/BitPermTable.cpp:19-34)."""
    v = np.asarray(values, np.int64).copy()
    for p in sorted(positions):
        lo = v & ((1 << p) - 1)
        v = ((v >> p) << (p + 1)) | lo
    return v


class SamplingPool:
    """cumprob = prefix sum of prob normalised by its total, error if the
    total is more than 0.05 from 1; sample = upper_bound(cumprob, u) with
    empty-lane bits inserted: qgate/simulator/src/CPUSamplingPool.cpp:8-81,
    qgate/simulator/pyruntime.py:278-321."""

    def __init__(self, prob, empty_lanes=()):
        prob = np.asarray(prob, np.float64)
        cum = np.cumsum(prob)
        total = cum[-1]
        if abs(total - 1.) > 0.05:
            raise RuntimeError('error in probability sum is beyond 0.05., %g.' % total)
        self.cumprob = cum * (1. / total)
        self.empty_lanes = list(empty_lanes)

    def sample(self, randnum):
        idx = np.searchsorted(self.cumprob, np.asarray(randnum, np.float64), side='right')
        idx = np.minimum(idx, self.cumprob.size - 1)
        if self.empty_lanes:
            idx = insert_zero_bits(idx, self.empty_lanes)
        return idx.astype(np.int64)


def boundary_tolerance_mask(cdf_ref, cdf_test, randnum):
    """Uniforms within tau = max|cdf_test - cdf_ref| of a CDF boundary of the
    reference: sampled indices may legitimately differ there."""
    tau = float(np.max(np.abs(np.asarray(cdf_ref) - np.asarray(cdf_test)))) if len(cdf_ref) else 0.
    u = np.asarray(randnum, np.float64)
    i = np.searchsorted(cdf_ref, u, side='right')
    lo = np.where(i > 0, np.asarray(cdf_ref)[np.maximum(i - 1, 0)], -np.inf)
    hi = np.asarray(cdf_ref)[np.minimum(i, len(cdf_ref) - 1)]
    return (np.abs(u - lo) <= tau) | (np.abs(u - hi) <= tau), tau


# ------------------------------------------------------------------ Pauli observables

def pauli_expectation(psi, x_mask, z_mask):
    """<psi|P|psi> for the Pauli string with X on x_mask & ~z_mask, Z on
    z_mask & ~x_mask and Y on x_mask & z_mask, built by applying the 2x2
    Pauli matrices (qgate/simulator/pymatrix.py:73-89).  The reference
    obtains Pr(+1) = (1 + <P>) / 2 of it by diagonalisation
    (qgate/model/pauli_gates_diagonalizer.py:96-135)."""
    n = int(psi.size).bit_length() - 1
    phi = psi.astype(np.complex128).copy()
    for q in range(n):
        xb, zb = (x_mask >> q) & 1, (z_mask >> q) & 1
        if xb and zb:
            apply_gate(phi, gate_matrix('Y'), q)
        elif xb:
            apply_gate(phi, gate_matrix('X'), q)
        elif zb:
            apply_gate(phi, gate_matrix('Z'), q)
    return float(np.vdot(psi.astype(np.complex128), phi).real)


# ------------------------------------------------------------------ circuits

def run_ops(n, ops, dtype=np.complex128, psi=None):
    """Runs a flat op list on one n-lane state.  ops: ('g', name, args, adj,
    target, controls) tuples, or ('m', dense_matrix, targets, controls)."""
    psi = initial_state(n, dtype) if psi is None else psi
    for op in ops:
        if op[0] == 'g':
            _, name, args, adj, target, controls = op
            apply_controlled_gate(psi, gate_matrix(name, args, adj), list(controls), target)
        elif op[0] == 'm':
            _, mat, targets, controls = op
            apply_matrix(psi, mat, list(targets), list(controls))
        else:
            raise ValueError(op[0])
    return psi
