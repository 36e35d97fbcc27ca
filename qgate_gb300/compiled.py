"""Compiled circuits: a gate list handed to the engine once and applied in one
call, optionally replayed from a captured CUDA graph.

The reference front-end drives its runtime one gate per call: the model
executor turns every `model.Gate` of a preprocessed circuit into a runtime
operator (qgate/simulator/model_executor.py:151-166) and the operator
executor calls `apply_gate` / `apply_controlled_gate` for each one
(qgate/simulator/rop_executor.py:28-34).  `CompiledCircuit` takes the same
per-gate information -- gate type, adjoint flag, local target lane, local
control lanes -- as one table, so a run is one call with no per-gate Python
or FFI work.  With `graph=True` the first run on a state buffer plans the
fused stages and captures their launches into a CUDA graph; later runs on the
same buffer replay the graph, without host planning.

    circ = CompiledCircuit(np.float32, [(H(), False, 0, []), (X(), False, 1, [0])])
    circ.run(qstates)        # same result as the two apply_* calls
"""
import ctypes

import numpy as np

from . import _native as nat
from .gb300runtime import _matrix_entry, _prec


def _matrix8(gate, adjoint):
    """8 doubles (row-major, interleaved re/im) of a gate type or of a 2x2
    complex matrix given directly."""
    if isinstance(gate, np.ndarray):
        m = np.asarray(gate, np.complex128)
        if m.shape != (2, 2):
            raise ValueError('a gate matrix must be 2x2, got {}.'.format(m.shape))
        if adjoint:
            m = m.conj().T
        return np.stack([m.real, m.imag], axis=-1).reshape(-1)
    return _matrix_entry(gate, adjoint)[0]


class CompiledCircuit:
    """gates: iterable of (gate, adjoint, target_lane, control_lanes), the
    arguments of the runtime's apply_gate / apply_controlled_gate; `gate` is
    a qgate gate type or a 2x2 complex matrix (numpy array)."""

    def __init__(self, dtype, gates, graph=True):
        targets, offsets, ctrls, mats = [], [0], [], []
        for gate, adjoint, target, controls in gates:
            targets.append(int(target))
            ctrls.extend(int(c) for c in controls)
            offsets.append(len(ctrls))
            mats.append(_matrix8(gate, adjoint))
        self.n_gates = len(targets)
        t = nat.int_array(targets)
        o = nat.int_array(offsets)
        c = nat.int_array(ctrls)
        m = np.ascontiguousarray(np.asarray(mats, np.float64).reshape(-1))
        if m.size == 0:
            m = np.zeros(8, np.float64)
        self.ptr = nat.new_handle('qg_circuit_new', _prec(dtype), self.n_gates, nat.as_iptr(t),
                                  nat.as_iptr(o), nat.as_iptr(c) if c.size else None,
                                  nat.as_dptr(m))
        self.graph = bool(graph)
        if self.graph:
            nat.call('qg_circuit_set_graph', self.ptr, 1)

    def run(self, qstates):
        """Applies the circuit to `qstates` (asynchronously, like apply_gate)."""
        nat.call('qg_circuit_run', self.ptr, qstates.ptr)

    def set_graph(self, on):
        nat.call('qg_circuit_set_graph', self.ptr, 1 if on else 0)
        self.graph = bool(on)

    def stats(self):
        """(whether a CUDA graph is captured, HBM passes of one run)."""
        cap = ctypes.c_int(0)
        passes = ctypes.c_int64(0)
        nat.call('qg_circuit_stats', self.ptr, ctypes.byref(cap), ctypes.byref(passes))
        return bool(cap.value), int(passes.value)

    def delete(self):
        if self.ptr:
            nat.call('qg_circuit_delete', self.ptr)
            self.ptr = 0

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.delete()
