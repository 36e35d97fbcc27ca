"""ctypes binding of libqgate_gb300.so (the C ABI in include/qgate_gb300.h).

The shared library is built in-tree by `qgate_gb300.csrc.build`.  There is no
fallback: if the library is missing or cannot be loaded, importing this
module raises, so nothing can silently run on the CPU instead of the GPU.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, 'libqgate_gb300.so')

QG_OK, QG_ERR_VALUE, QG_ERR_RUNTIME, QG_ERR_CUDA, QG_ERR_NOMEM, QG_ERR_TIMEOUT = range(6)
PREC_FP64, PREC_FP32 = 1, 2
MATHOP_NULL, MATHOP_PROB = 0, 1

_h = ctypes.c_uint64
_hp = ctypes.POINTER(ctypes.c_uint64)
_i = ctypes.c_int
_i64 = ctypes.c_int64
_u64 = ctypes.c_uint64
_d = ctypes.c_double
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_i64p = ctypes.POINTER(ctypes.c_int64)
_vp = ctypes.c_void_p

# name -> argtypes; every entry point returns int status.
SIGNATURES = {
    'qg_devices_initialize': [_i, _i64],
    'qg_devices_clear': [],
    'qg_arena_stats': [_i64p, _i64p],
    'qg_qubit_states_new': [_i, _hp],
    'qg_qubit_states_delete': [_h],
    'qg_qubit_states_deallocate': [_h],
    'qg_qubit_states_get_n_lanes': [_h, _ip],
    'qg_qubit_processor_new': [_i, _hp],
    'qg_qubit_processor_delete': [_h],
    'qg_qubit_processor_synchronize': [_h],
    'qg_qubit_processor_reset': [_h],
    'qg_qubit_processor_initialize_qubit_states': [_h, _h, _i],
    'qg_qubit_processor_reset_qubit_states': [_h, _h],
    'qg_qubit_processor_calc_probability': [_h, _h, _i, _dp],
    'qg_qubit_processor_join': [_h, _h, _hp, _i, _i],
    'qg_qubit_processor_decohere': [_h, _i, _d, _h, _i],
    'qg_qubit_processor_decohere_and_separate': [_h, _i, _d, _h, _h, _h, _i],
    'qg_qubit_processor_apply_reset': [_h, _h, _i],
    # per-gate entry points take raw addresses (ints) for speed
    'qg_qubit_processor_apply_gate': [_h, _vp, _h, _i],
    'qg_qubit_processor_apply_controlled_gate': [_h, _vp, _h, _vp, _i, _i],
    'qg_circuit_new': [_i, _i, _ip, _ip, _ip, _dp, _hp],
    'qg_circuit_set_graph': [_h, _i],
    'qg_circuit_run': [_h, _h],
    'qg_circuit_stats': [_h, _ip, _i64p],
    'qg_circuit_delete': [_h],
    'qg_qubit_processor_apply_multi': [_h, _dp, _h, _ip, _i, _ip, _i],
    'qg_qubit_processor_calc_pauli_expectation': [_h, _h, _u64, _u64, _dp],
    'qg_qubit_processor_calc_norm': [_h, _h, _dp],
    'qg_set_fusion': [_i],
    'qg_set_fusion_params': [_i, _i, _i, _i],
    'qg_set_stage_pipelining': [_i],
    'qg_set_trace_replay': [_i],
    'qg_set_batch_one_launch': [_i],
    'qg_grouping_stats': [_i64p, _i, _i],
    'qg_trace_stats': [_i64p, _i64p, _i],
    'qg_set_tensor_blocks': [_i],
    'qg_tensor_stage_status': [_i, _ip],
    'qg_set_host_direct': [_i],
    'qg_set_pageable_copy': [_i],
    'qg_set_pool_guide_index_shift': [_i],
    'qg_gate_stats': [_i64p, _i64p, _i64p, _i],
    'qg_timing_enable': [_i],
    'qg_timing_read': [ctypes.c_char_p, _i64p, _dp, _i],
    'qg_get_stream': [ctypes.POINTER(ctypes.c_uint64)],
    'qg_device_info': [_i64p, _i],
    'qg_qubit_states_get_raw': [_h, _vp, _i64],
    'qg_qubit_states_set_raw': [_h, _vp, _i64],
    'qg_gate_matrix': [ctypes.c_char_p, _vp, _i, _i, _vp],
    'qg_calc_probability_noalloc': [_i, _vp, _i, _i, _vp, _u64],
    'qg_adjoint_expectation': [_i, _i, _vp, _i, _vp, _i, _i, _vp, _i, _i, _vp, _vp],
    'qg_batch_sum_z': [_i, _i, _vp, _vp, _vp, _vp],
    'qg_qubits_states_getter_new': [_i, _hp],
    'qg_qubits_states_getter_delete': [_h],
    'qg_qubits_states_getter_get_states': [_h, _vp, _i64, _i, _ip, _ip, _hp, _i, _u64, _i,
                                           _i64, _i64, _i64],
    'qg_qubits_states_getter_prepare_prob_array': [_h, _vp, _ip, _ip, _hp, _i, _i, _i],
    'qg_qubits_states_getter_create_sampling_pool': [_h, _ip, _ip, _hp, _i, _i, _i, _ip, _i,
                                                     _hp],
    'qg_sampling_pool_sample': [_h, _i64p, _i64, _dp],
    'qg_sampling_pool_delete': [_h],
}


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError('libqgate_gb300.so not built (%s); run '
                          '`python -c "import __graft_entry__ as g; g.build()"` or '
                          '`python -m qgate_gb300.csrc.build`' % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, argtypes in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = ctypes.c_int
    lib.qg_last_error.argtypes = []
    lib.qg_last_error.restype = ctypes.c_char_p
    return lib


lib = _load()


def check(status):
    if status == QG_OK:
        return
    msg = lib.qg_last_error().decode(errors='replace')
    if status == QG_ERR_VALUE:
        raise ValueError(msg)
    if status == QG_ERR_NOMEM:
        raise MemoryError(msg)
    raise RuntimeError(msg)


def call(name, *args):
    check(getattr(lib, name)(*args))


def new_handle(name, *args):
    h = ctypes.c_uint64(0)
    check(getattr(lib, name)(*args, ctypes.byref(h)))
    return h.value


def as_dptr(a):
    return a.ctypes.data_as(_dp)


def as_iptr(a):
    return a.ctypes.data_as(_ip)


def int_array(values):
    return np.ascontiguousarray(np.asarray(values, dtype=np.int32).reshape(-1))


def handle_array(values):
    return np.ascontiguousarray(np.asarray(values, dtype=np.uint64).reshape(-1))


def gate_matrix(name, args=(), adjoint=False):
    """2x2 complex128 matrix of a named gate (conventions of the reference's
    qgate/simulator/src/GateMatrix.cpp:13-158)."""
    a = np.ascontiguousarray(np.asarray(args, dtype=np.float64).reshape(-1))
    out = np.empty(8, np.float64)
    check(lib.qg_gate_matrix(name.encode(), a.ctypes.data if a.size else None, int(a.size),
                             1 if adjoint else 0, out.ctypes.data))
    return out.view(np.complex128).reshape(2, 2)


def set_fusion(max_tile_lanes):
    call('qg_set_fusion', int(max_tile_lanes))


def set_fusion_params(prec, tile_lanes, reg_lanes, cost_budget=0):
    call('qg_set_fusion_params', int(prec), int(tile_lanes), int(reg_lanes), int(cost_budget))


def set_tensor_blocks(on):
    """Run complex64 stages of 12/13-lane tiles as fused 5-lane blocks on the
    tensor cores (tcgen05 kind::f16 on split FP16 operands)."""
    call('qg_set_tensor_blocks', 1 if on else 0)


def set_trace_replay(on):
    """Replay recurring runs of per-gate calls from captured CUDA graphs."""
    call('qg_set_trace_replay', 1 if on else 0)


def trace_stats(reset=False):
    """{'hits': graph replays, 'captures': runs captured} of trace replay."""
    h, c = _i64(0), _i64(0)
    check(lib.qg_trace_stats(ctypes.byref(h), ctypes.byref(c), 1 if reset else 0))
    return {'hits': h.value, 'captures': c.value}


GROUPING_KEYS = ('joins', 'krons', 'allocs', 'separates', 'inplace', 'copies', 'cow')


def grouping_stats(reset=False):
    """Counters of the qubit-grouping policy: join calls, kron passes, state
    buffers allocated, decohere_and_separate calls, separations formed in
    place / by copy, copies of buffers still read by a lazy object."""
    out = np.zeros(len(GROUPING_KEYS), np.int64)
    check(lib.qg_grouping_stats(out.ctypes.data_as(_i64p), len(out), 1 if reset else 0))
    return dict(zip(GROUPING_KEYS, (int(x) for x in out)))


def tensor_stage_status(reset=False):
    v = ctypes.c_int(0)
    check(lib.qg_tensor_stage_status(1 if reset else 0, ctypes.byref(v)))
    return v.value


def gate_stats(reset=False):
    g, p, b = _i64(0), _i64(0), _i64(0)
    check(lib.qg_gate_stats(ctypes.byref(g), ctypes.byref(p), ctypes.byref(b), 1 if reset else 0))
    return {'gates': g.value, 'passes': p.value, 'bytes': b.value}


def timing_enable(on=True):
    call('qg_timing_enable', 1 if on else 0)


def timing_read(kernel_class, reset=False):
    n, ms = _i64(0), _d(0.)
    check(lib.qg_timing_read(kernel_class.encode(), ctypes.byref(n), ctypes.byref(ms),
                             1 if reset else 0))
    return n.value, ms.value


KERNEL_CLASSES = ('stage', 'tstage', 'gate', 'multi', 'init', 'prob', 'pauli', 'measure', 'join',
                  'gather', 'marginal', 'scan', 'search', 'batch')


def timing_all(reset=False):
    out = {}
    for k in KERNEL_CLASSES:
        out[k] = timing_read(k)
    if reset:
        timing_read('', reset=True)
    return out


DEVICE_INFO_KEYS = ('sm_count', 'smem_optin_per_block', 'l2_bytes', 'pageable_memory_access',
                    'pageable_uses_host_page_tables', 'concurrent_managed_access', 'cc_major',
                    'cc_minor', 'sm_clock_khz', 'mem_clock_khz', 'free_bytes', 'total_bytes')


def device_info():
    buf = np.zeros(len(DEVICE_INFO_KEYS), np.int64)
    check(lib.qg_device_info(buf.ctypes.data_as(_i64p), len(buf)))
    return dict(zip(DEVICE_INFO_KEYS, (int(v) for v in buf)))


def stream_handle():
    s = ctypes.c_uint64(0)
    check(lib.qg_get_stream(ctypes.byref(s)))
    return s.value


def arena_stats():
    a, b = _i64(0), _i64(0)
    check(lib.qg_arena_stats(ctypes.byref(a), ctypes.byref(b)))
    return {'in_use': a.value, 'cached': b.value}
