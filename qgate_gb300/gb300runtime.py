"""GB300 runtime module for the qgate simulator front-end.

This module is a drop-in runtime package ("defpkg") for the reference's
`Simulator(defpkg, **prefs)` (qgate/simulator/simulator.py:13-23): it
exports `create_qubit_states(dtype)` and `create_qubits_states_getter(dtype)`
and returns objects with the method sets of the reference's native wrappers
(qgate/simulator/native_qubit_processor.py:6-59,
qgate/simulator/native_qubit_states.py:4-33,
qgate/simulator/native_qubits_states_getter.py:6-102,
qgate/simulator/native_sampling_pool.py:5-24), and the module-level
preference / finalisation calls of qgate/simulator/cudaruntime.py:26-91.

    import qgate, qgate_gb300.gb300runtime as rt
    sim = qgate.simulator.simulator.Simulator(rt, dtype=np.float32)

Every call goes through the C ABI of libqgate_gb300.so to sm_103a kernels;
there is no CPU code path.
"""
import atexit
import sys
import weakref

import numpy as np

from . import _native as nat
from .observation import ObservationList

this = sys.modules[__name__]
this.initialized = False
this.native_instances = weakref.WeakValueDictionary()
this.device_ids = []
this.memory_store_size = -1


def _prec(dtype):
    if dtype == np.float64:
        return nat.PREC_FP64
    if dtype == np.float32:
        return nat.PREC_FP32
    raise RuntimeError('unexpected dtype, {}.'.format(dtype))


def set_preference(device_ids=[], max_po2idx_per_chunk=-1, memory_store_size=-1):
    """Mirror of cudaruntime.set_preference (qgate/simulator/cudaruntime.py:33-41).

    One GPU holds the whole state, so `device_ids` may name a single device
    (repeats of it are accepted) and `max_po2idx_per_chunk` is ignored;
    `memory_store_size` caps the device arena in bytes."""
    if this.initialized:
        raise RuntimeError('already initialized.')
    ids = sorted(set(device_ids))
    if len(ids) > 1:
        raise RuntimeError('the GB300 runtime uses one GPU; got device_ids {}.'.format(device_ids))
    if len(ids) != 0:
        this.device_ids = ids
    if memory_store_size != -1:
        this.memory_store_size = memory_store_size


def reset_preference(device_ids=[], max_po2idx_per_chunk=-1, memory_store_size=-1):
    this.device_ids = []
    this.memory_store_size = -1


def module_init():
    dev = this.device_ids[0] if this.device_ids else -1
    nat.call('qg_devices_initialize', int(dev), int(this.memory_store_size))
    this.initialized = True


def module_finalize():
    for obj in list(this.native_instances.values()):
        obj.delete()
    if this.initialized:
        nat.call('qg_devices_clear')
    this.initialized = False


atexit.register(module_finalize)


# ---------------------------------------------------------------- gate matrices

_matrix_cache = {}
_name_bytes = {}
_ctrl_cache = {}
_gate_matrix_fn = nat.lib.qg_gate_matrix
_apply_gate_fn = nat.lib.qg_qubit_processor_apply_gate
_apply_controlled_fn = nat.lib.qg_qubit_processor_apply_controlled_gate


def _matrix_entry(gate_type, adjoint):
    """(matrix, its address): the 2x2 complex128 matrix of a gate type as 8
    contiguous doubles, cached per (class, args, adjoint)."""
    cls = type(gate_type)
    args = getattr(gate_type, 'args', ())
    key = (cls, tuple(args), bool(adjoint))
    e = _matrix_cache.get(key)
    if e is None:
        name = _name_bytes.get(cls)
        if name is None:
            name = _name_bytes.setdefault(cls, cls.__name__.encode())
        a = np.asarray(args, np.float64).reshape(-1)
        m = np.empty(8, np.float64)
        nat.check(_gate_matrix_fn(name, a.ctypes.data if a.size else None, a.size,
                                  1 if adjoint else 0, m.ctypes.data))
        if len(_matrix_cache) > 4096:
            _matrix_cache.clear()
        e = _matrix_cache[key] = (m, m.ctypes.data)
    return e


def gate_matrix(gate_type, adjoint):
    """2x2 complex128 matrix of a qgate gate type, as 8 contiguous doubles.

    The reference builds it from the `cmatf` factory registered per gate
    class (qgate/simulator/cpumatrix.py:4-20, qgate/simulator/src/glue.cpp:383-395);
    here the class name and `args` select the same formulas in the C ABI."""
    return _matrix_entry(gate_type, adjoint)[0]


def _controls(lanes):
    """(int32 array, address) of a control-lane list, cached per tuple."""
    key = tuple(lanes)
    e = _ctrl_cache.get(key)
    if e is None:
        a = nat.int_array(key)
        if len(_ctrl_cache) > 4096:
            _ctrl_cache.clear()
        e = _ctrl_cache[key] = (a, a.ctypes.data)
    return e


# ---------------------------------------------------------------- processor / states

class GB300QubitProcessor:
    def __init__(self, dtype, ptr):
        self.dtype = dtype
        self.ptr = ptr

    def __del__(self):
        self.delete()

    def delete(self):
        if hasattr(self, 'ptr'):
            nat.lib.qg_qubit_processor_delete(self.ptr)
            del self.ptr

    def synchronize(self):
        nat.call('qg_qubit_processor_synchronize', self.ptr)

    def reset(self):
        nat.call('qg_qubit_processor_reset', self.ptr)

    def initialize_qubit_states(self, qstates, n_lanes):
        nat.call('qg_qubit_processor_initialize_qubit_states', self.ptr, qstates.ptr, int(n_lanes))
        qstates.reset_lane_states()

    def reset_qubit_states(self, qstates):
        nat.call('qg_qubit_processor_reset_qubit_states', self.ptr, qstates.ptr)
        qstates.reset_lane_states()

    def calc_probability(self, qstates, local_lane):
        out = nat._d(0.)
        nat.call('qg_qubit_processor_calc_probability', self.ptr, qstates.ptr, int(local_lane),
                 nat.ctypes.byref(out))
        return out.value

    def join(self, qstates, qstates_list, n_new_qregs):
        ptrs = nat.handle_array([qs.ptr for qs in qstates_list])
        nat.call('qg_qubit_processor_join', self.ptr, qstates.ptr,
                 ptrs.ctypes.data_as(nat._hp), len(ptrs), int(n_new_qregs))

    def decohere(self, value, prob, qstates, local_lane):
        nat.call('qg_qubit_processor_decohere', self.ptr, int(value), float(prob), qstates.ptr,
                 int(local_lane))
        return value

    def decohere_and_separate(self, value, prob, qstates0, qstates1, qstates, local_lane):
        nat.call('qg_qubit_processor_decohere_and_separate', self.ptr, int(value), float(prob),
                 qstates0.ptr, qstates1.ptr, qstates.ptr, int(local_lane))
        return value

    def apply_reset(self, qstates, local_lane):
        nat.call('qg_qubit_processor_apply_reset', self.ptr, qstates.ptr, int(local_lane))

    def apply_gate(self, gate_type, _adjoint, qstates, local_lane):
        st = _apply_gate_fn(self.ptr, _matrix_entry(gate_type, _adjoint)[1], qstates.ptr,
                            int(local_lane))
        if st:
            nat.check(st)

    def apply_controlled_gate(self, gate_type, _adjoint, qstates, local_control_lanes,
                              local_target_lane):
        ctrl, addr = _controls(local_control_lanes)
        st = _apply_controlled_fn(self.ptr, _matrix_entry(gate_type, _adjoint)[1], qstates.ptr,
                                  addr, len(ctrl), int(local_target_lane))
        if st:
            nat.check(st)

    # ---- extensions (no counterpart in the reference runtime protocol)

    def apply_matrix(self, mat, qstates, target_lanes, local_control_lanes=()):
        """Dense 2^k x 2^k gate on k target lanes (targets[0] = matrix bit 0)."""
        mat = np.ascontiguousarray(np.asarray(mat, np.complex128))
        k = len(target_lanes)
        if mat.shape != (1 << k, 1 << k):
            raise ValueError('matrix shape {} does not match {} targets.'.format(mat.shape, k))
        t = nat.int_array(target_lanes)
        c = nat.int_array(local_control_lanes)
        flat = mat.reshape(-1).view(np.float64)
        nat.call('qg_qubit_processor_apply_multi', self.ptr, nat.as_dptr(flat), qstates.ptr,
                 nat.as_iptr(t), len(t), nat.as_iptr(c) if len(c) else None, len(c))

    def calc_pauli_expectation(self, qstates, x_mask, z_mask):
        out = nat._d(0.)
        nat.call('qg_qubit_processor_calc_pauli_expectation', self.ptr, qstates.ptr,
                 int(x_mask), int(z_mask), nat.ctypes.byref(out))
        return out.value

    def calc_norm(self, qstates):
        out = nat._d(0.)
        nat.call('qg_qubit_processor_calc_norm', self.ptr, qstates.ptr, nat.ctypes.byref(out))
        return out.value


class GB300QubitStates:
    def __init__(self, ptr, processor):
        self.ptr = ptr
        self.processor = processor

    def __del__(self):
        self.delete()

    def delete(self):
        if hasattr(self, 'ptr'):
            nat.lib.qg_qubit_states_delete(self.ptr)
            del self.ptr
        if hasattr(self, 'processor'):
            self.processor.delete()
            del self.processor

    def get_n_lanes(self):
        n = nat._i(0)
        nat.call('qg_qubit_states_get_n_lanes', self.ptr, nat.ctypes.byref(n))
        return n.value

    def reset_lane_states(self):
        self.lane_states = [-1] * self.get_n_lanes()

    def get_lane_state(self, lane):
        return self.lane_states[lane]

    def set_lane_state(self, lane, value):
        self.lane_states[lane] = value

    def calc_probability(self, lane):
        return self.processor.calc_probability(self, lane)

    # ---- extensions

    def get_raw(self):
        """All 2^n amplitudes in local lane order (complex64/complex128)."""
        dtype = np.complex128 if self.processor.dtype == np.float64 else np.complex64
        out = np.empty(1 << self.get_n_lanes(), dtype)
        nat.call('qg_qubit_states_get_raw', self.ptr, out.ctypes.data, out.size)
        return out

    def set_raw(self, values):
        dtype = np.complex128 if self.processor.dtype == np.float64 else np.complex64
        v = np.ascontiguousarray(np.asarray(values, dtype))
        nat.call('qg_qubit_states_set_raw', self.ptr, v.ctypes.data, v.size)


def create_qubit_states(dtype):
    if not this.initialized:
        module_init()
    prec = _prec(dtype)
    proc = GB300QubitProcessor(dtype, nat.new_handle('qg_qubit_processor_new', prec))
    this.native_instances[id(proc)] = proc
    qstates = GB300QubitStates(nat.new_handle('qg_qubit_states_new', prec), proc)
    this.native_instances[id(qstates)] = qstates
    return qstates


# ---------------------------------------------------------------- getter / pool

def _mathop_code(mathop):
    name = getattr(mathop, '__name__', None)
    if name == 'null':
        return nat.MATHOP_NULL
    if name == 'abs2':
        return nat.MATHOP_PROB
    raise RuntimeError('unknown math operation, {}'.format(str(mathop)))


def _translate(lane_trans):
    """lane_trans [(qstates, [Lane(local, external)])] -> C tables.

    Same translation as qgate/simulator/native_qubits_states_getter.py:84-95."""
    ptrs, tables, counts = [], [], []
    for qstates, lanelist in lane_trans:
        ptrs.append(qstates.ptr)
        table = [None] * len(lanelist)
        for lane in lanelist:
            table[lane.local] = lane.external
        tables.extend(table)
        counts.append(len(table))
    return nat.handle_array(ptrs), nat.int_array(tables), nat.int_array(counts)


def _lane_mask(lanes):
    mask = 0
    for pos in lanes:
        mask |= 1 << pos
    return mask


class GB300SamplingPool:
    def __init__(self, ptr, qreg_ordering, mask):
        self.ptr = ptr
        self.qreg_ordering = qreg_ordering
        self.mask = mask

    def __del__(self):
        self.delete()

    def delete(self):
        if hasattr(self, 'ptr'):
            nat.lib.qg_sampling_pool_delete(self.ptr)
            del self.ptr

    def sample(self, n_samples, randnum=None):
        obs = np.empty([n_samples], np.int64)
        if randnum is None:
            randnum = np.random.random_sample([n_samples])
        u = np.ascontiguousarray(np.asarray(randnum, np.float64).reshape(-1))
        if u.size < n_samples:
            raise ValueError('array size too small.')
        nat.call('qg_sampling_pool_sample', self.ptr, obs.ctypes.data_as(nat._i64p),
                 int(n_samples), nat.as_dptr(u))
        return ObservationList(self.qreg_ordering, obs, self.mask)


class GB300QubitsStatesGetter:
    def __init__(self, dtype, ptr):
        self.dtype = dtype
        self.ptr = ptr

    def __del__(self):
        self.delete()

    def delete(self):
        if hasattr(self, 'ptr'):
            nat.lib.qg_qubits_states_getter_delete(self.ptr)
            del self.ptr

    def get_states(self, values, offset, mathop, lane_trans, empty_lanes, n_states, start, step):
        code = _mathop_code(mathop)
        n_lanes = sum([len(lanepos_list) for qstates, lanepos_list in lane_trans])
        n_qregs = n_lanes + len(empty_lanes)
        if values.ndim != 1 or not values.flags['C_CONTIGUOUS']:
            raise ValueError('values must be a contiguous 1-d array.')
        if len(values) - offset < n_states:
            raise ValueError('array size too small.')
        expected = {(nat.MATHOP_NULL, np.float64): np.complex128,
                    (nat.MATHOP_NULL, np.float32): np.complex64,
                    (nat.MATHOP_PROB, np.float64): np.float64,
                    (nat.MATHOP_PROB, np.float32): np.float32}[(code, self.dtype)]
        if values.dtype != expected:
            raise ValueError('values dtype {} != {}.'.format(values.dtype, np.dtype(expected)))
        ptrs, tables, counts = _translate(lane_trans)
        nat.call('qg_qubits_states_getter_get_states', self.ptr, values.ctypes.data, int(offset),
                 code, nat.as_iptr(tables) if tables.size else None,
                 nat.as_iptr(counts) if counts.size else None,
                 ptrs.ctypes.data_as(nat._hp) if ptrs.size else None, len(ptrs),
                 _lane_mask(empty_lanes), int(n_qregs), int(n_states), int(start), int(step))

    def create_sampling_pool(self, qreg_ordering, n_lanes, n_hidden_lanes, lane_trans,
                             empty_lanes, sampling_pool_factory=None):
        # Hidden lanes go above the pool lanes, as in the reference's CUDA
        # runtime (qgate/simulator/cudaruntime.py:64-72).
        hidden_idx = n_lanes
        for qs, lanelist in lane_trans:
            for lane in lanelist:
                if lane.external == -1:
                    lane.external = hidden_idx
                    hidden_idx += 1
        ptrs, tables, counts = _translate(lane_trans)
        if sampling_pool_factory is not None:
            prob = np.empty([1 << n_lanes], self.dtype)
            nat.call('qg_qubits_states_getter_prepare_prob_array', self.ptr, prob.ctypes.data,
                     nat.as_iptr(tables), nat.as_iptr(counts), ptrs.ctypes.data_as(nat._hp),
                     len(ptrs), int(n_lanes), int(n_hidden_lanes))
            return sampling_pool_factory(prob, empty_lanes, qreg_ordering)
        el = nat.int_array(empty_lanes)
        ptr = nat.new_handle('qg_qubits_states_getter_create_sampling_pool', self.ptr,
                             nat.as_iptr(tables), nat.as_iptr(counts),
                             ptrs.ctypes.data_as(nat._hp), len(ptrs), int(n_lanes),
                             int(n_hidden_lanes), nat.as_iptr(el) if el.size else None, len(el))
        pool = GB300SamplingPool(ptr, qreg_ordering, _lane_mask(empty_lanes))
        this.native_instances[id(pool)] = pool
        return pool


def create_qubits_states_getter(dtype):
    if not this.initialized:
        module_init()
    getter = GB300QubitsStatesGetter(dtype, nat.new_handle('qg_qubits_states_getter_new',
                                                           _prec(dtype)))
    this.native_instances[id(getter)] = getter
    return getter
