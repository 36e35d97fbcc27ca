"""ctypes loader for the oracle's compiled C port (oracle/cpu_statevec.c).

TEST INFRASTRUCTURE ONLY: used by tests, smoke() and bench.py's CPU-baseline
and reference arms; never by the product.  `build()` compiles the port with
the host gcc into oracle/_build/ (the GPU host builds its own copy)."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, 'cpu_statevec.c')
LIB = os.path.join(HERE, '_build', 'libcpu_statevec.so')

_lib = None


def build(force=False):
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        subprocess.run(['gcc', '-O3', '-fopenmp', '-fPIC', '-shared', SRC, '-o', LIB, '-lm'],
                       check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, i, d, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_longlong
        L.cs_num_threads.restype = i
        L.cs_init_basis.argtypes = [vp, i, i]
        L.cs_apply_gate.argtypes = [vp, i, i, vp, vp, i, i]
        L.cs_calc_probability.argtypes = [vp, i, i, i]
        L.cs_calc_probability.restype = d
        L.cs_probabilities.argtypes = [vp, i, i, vp]
        L.cs_prefix_sum_normalise.argtypes = [vp, i64]
        L.cs_prefix_sum_normalise.restype = d
        L.cs_sample.argtypes = [vp, i64, vp, vp, i64, vp, i]
        L.cs_run_circuit.argtypes = [vp, i, i, i, vp, vp, vp, vp, i]
        L.cs_run_circuit.restype = i
        _lib = L
    return _lib


def num_threads():
    return lib().cs_num_threads()


class State:
    """A 2^n state in host memory driven by the C port."""

    def __init__(self, n, dtype=np.complex64):
        self.n = n
        self.prec = 1 if dtype == np.complex128 else 2
        self.psi = np.empty(1 << n, dtype)
        lib().cs_init_basis(self.psi.ctypes.data, n, self.prec)

    def apply(self, mat, target, controls=()):
        m = np.ascontiguousarray(np.asarray(mat, np.complex128).reshape(-1)).view(np.float64)
        c = np.ascontiguousarray(np.asarray(controls, np.int32))
        lib().cs_apply_gate(self.psi.ctypes.data, self.n, self.prec, m.ctypes.data,
                            c.ctypes.data if c.size else None, int(c.size), int(target))

    def run(self, gates, max_lanes=14):
        """Applies [(2x2 matrix, target, controls)] in order, in cache-sized
        passes (cs_run_circuit: the same result as one apply() per gate).
        Returns the number of passes."""
        mats = np.ascontiguousarray(np.array([np.asarray(m, np.complex128).reshape(4)
                                              for m, _, _ in gates]).reshape(-1)).view(np.float64)
        targets = np.ascontiguousarray([t for _, t, _ in gates], np.int32)
        off = np.zeros(len(gates) + 1, np.int32)
        off[1:] = np.cumsum([len(c) for _, _, c in gates])
        ctrls = np.ascontiguousarray([q for _, _, c in gates for q in c] or [0], np.int32)
        r = lib().cs_run_circuit(self.psi.ctypes.data, self.n, self.prec, len(gates),
                                 mats.ctypes.data, targets.ctypes.data, off.ctypes.data,
                                 ctrls.ctypes.data, max_lanes)
        if r < 0:
            raise ValueError('max_lanes must be in [5, 20]')
        return r

    def calc_probability(self, lane):
        return lib().cs_calc_probability(self.psi.ctypes.data, self.n, self.prec, lane)

    def probabilities(self):
        out = np.empty(1 << self.n, np.float64)
        lib().cs_probabilities(self.psi.ctypes.data, self.n, self.prec, out.ctypes.data)
        return out


def prefix_cdf(prob, copy=True):
    """(cdf, total): the reference pool's normalised FP64 prefix sums of
    `prob` (cs_prefix_sum_normalise); copy=False overwrites a contiguous
    float64 `prob` in place."""
    cdf = np.array(prob, np.float64) if copy else np.ascontiguousarray(prob, np.float64)
    total = lib().cs_prefix_sum_normalise(cdf.ctypes.data, cdf.size)
    return cdf, total


def sample_cdf(cdf, u, empty_lanes=()):
    """Indices the reference pool draws for uniforms `u` from a normalised
    CDF (cs_sample: upper_bound, clamped, empty-lane bits inserted)."""
    u = np.ascontiguousarray(u, np.float64)
    obs = np.empty(u.size, np.int64)
    e = np.ascontiguousarray(np.asarray(empty_lanes, np.int32))
    lib().cs_sample(cdf.ctypes.data, cdf.size, u.ctypes.data, obs.ctypes.data, u.size,
                    e.ctypes.data if e.size else None, int(e.size))
    return obs


def sampling_pool_sample(prob, u, empty_lanes=()):
    cdf = np.array(prob, np.float64)
    total = lib().cs_prefix_sum_normalise(cdf.ctypes.data, cdf.size)
    if abs(total - 1.) > 0.05:
        raise RuntimeError('error in probability sum is beyond 0.05., %g.' % total)
    u = np.ascontiguousarray(u, np.float64)
    obs = np.empty(u.size, np.int64)
    e = np.ascontiguousarray(np.asarray(empty_lanes, np.int32))
    lib().cs_sample(cdf.ctypes.data, cdf.size, u.ctypes.data, obs.ctypes.data, u.size,
                    e.ctypes.data if e.size else None, int(e.size))
    return obs
