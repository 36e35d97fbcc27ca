"""Replays a recorded boundary trace (tests/golden/traces/*.json) against a
runtime module and checks every observable result against the reference's.

A trace is the sequence of runtime-protocol calls that the reference
front-end (`qgate.simulator.Simulator`) made while running a scenario on the
reference's own C++ CPU runtime in complex128, with that runtime's results.
Replaying it against the GB300 runtime exercises the exact call pattern of
the reference front-end (gates, controlled gates, joins, measurements with
fixed outcomes, resets, gathers with lane permutations / empty lanes /
slices, sampling pools with hidden and empty lanes) without needing the
front-end itself.
"""
import json
import os

import numpy as np

from qgate_gb300.circuit import Lane, null, abs2  # noqa: F401
from qgate_gb300.circuit import gate_type as _gate_type

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
TRACE_DIR = os.path.join(GOLDEN, 'traces')


def trace_names():
    return sorted(f[:-5] for f in os.listdir(TRACE_DIR) if f.endswith('.json'))


def load_trace(name):
    with open(os.path.join(TRACE_DIR, name + '.json')) as f:
        t = json.load(f)
    arrays = dict(np.load(os.path.join(TRACE_DIR, name + '.npz')))
    return t['calls'], arrays


def make_gate_type(name, args):
    """A stand-in for a qgate GateType: its class name and `args` are what the
    runtimes read (qgate/simulator/cpumatrix.py, qgate/model/gate_type.py)."""
    return _gate_type(name, *args)


class Tolerance:
    def __init__(self, dtype):
        if dtype == np.float64:
            self.atol, self.rtol = 1e-11, 1e-9
        else:
            self.atol, self.rtol = 3e-6, 1e-4


class Stats:
    def __init__(self):
        self.max_err = 0.
        self.checks = 0
        self.samples = 0
        self.sample_mismatch = 0
        self.sample_mismatch_outside_tol = 0
        self.failures = []


def _close(stats, tol, what, got, want):
    got = np.asarray(got)
    want = np.asarray(want)
    stats.checks += 1
    if got.shape != want.shape:
        stats.failures.append('%s: shape %s != %s' % (what, got.shape, want.shape))
        return
    if got.size == 0:
        return
    err = float(np.max(np.abs(got.astype(np.complex128) - want.astype(np.complex128))))
    stats.max_err = max(stats.max_err, err)
    if not np.allclose(got, want, atol=tol.atol, rtol=tol.rtol):
        stats.failures.append('%s: max abs err %.3e' % (what, err))


def _lanes(lt, objs):
    return [(objs[sid], [Lane(l, e) for l, e in lanes]) for sid, lanes in lt]


def replay(calls, arrays, runtime, dtype):
    from oracle import statevec as sv
    tol = Tolerance(dtype)
    stats = Stats()
    objs = {}
    pools = {}
    getter = None
    last_qs = None
    for i, c in enumerate(calls):
        op = c[0]
        where = '#%d %s' % (i, op)
        if op == 'new_states':
            objs[c[1]] = runtime.create_qubit_states(dtype)
            last_qs = objs[c[1]]
        elif op == 'delete_states':
            qs = objs.pop(c[1], None)
            if qs is not None:
                if qs is last_qs:
                    last_qs = None
                if hasattr(qs, 'delete'):
                    qs.delete()
        elif op == 'new_getter':
            getter = objs[c[1]] = runtime.create_qubits_states_getter(dtype)
        elif op == 'init':
            qs = objs[c[1]]
            qs.processor.initialize_qubit_states(qs, c[2])
        elif op == 'reset_states':
            qs = objs[c[1]]
            qs.processor.reset_qubit_states(qs)
        elif op == 'prob':
            qs = objs[c[1]]
            _close(stats, tol, where, qs.processor.calc_probability(qs, c[2]), c[3])
        elif op == 'join':
            qs = objs[c[1]]
            qs.processor.join(qs, [objs[s] for s in c[2]], c[3])
        elif op == 'decohere':
            qs = objs[c[3]]
            qs.processor.decohere(c[1], c[2], qs, c[4])
        elif op == 'separate':
            qs = objs[c[5]]
            qs.processor.decohere_and_separate(c[1], c[2], objs[c[3]], objs[c[4]], qs, c[6])
        elif op == 'apply_reset':
            qs = objs[c[1]]
            qs.processor.apply_reset(qs, c[2])
        elif op == 'gate':
            _, name, args, adj, sid, target, ctrls = c
            qs = objs[sid]
            gt = make_gate_type(name, args)
            if ctrls:
                qs.processor.apply_controlled_gate(gt, adj, qs, ctrls, target)
            else:
                qs.processor.apply_gate(gt, adj, qs, target)
        elif op == 'sync':
            if last_qs is not None:
                last_qs.processor.synchronize()
        elif op == 'get_states':
            _, mathop, lt, empty, n_states, start, step, offset, length, key = c
            if mathop == 'null':
                vdtype = np.complex128 if dtype == np.float64 else np.complex64
                fn = null
            else:
                vdtype = dtype
                fn = abs2
            values = np.zeros(length, vdtype)
            getter.get_states(values, offset, fn, _lanes(lt, objs), empty, n_states, start, step)
            _close(stats, tol, where, values[offset:offset + n_states], arrays[key])
        elif op == 'pool':
            _, pid, ordering, n_lanes, n_hidden, lt, empty, has_factory, key = c
            captured = {}

            def factory(prob, empty_lanes, qreg_ordering):
                captured['prob'] = np.array(prob)
                return None
            getter.create_sampling_pool(ordering, n_lanes, n_hidden, _lanes(lt, objs), empty,
                                        factory)
            _close(stats, tol, where, captured['prob'], arrays[key])
            if not has_factory:
                pool = getter.create_sampling_pool(ordering, n_lanes, n_hidden,
                                                   _lanes(lt, objs), empty)
                ref_prob = arrays[key].astype(np.float64)
                cdf_ref = np.cumsum(ref_prob) / np.sum(ref_prob)
                eng = captured['prob'].astype(np.float64)
                cdf_eng = np.cumsum(eng) / np.sum(eng)
                pools[pid] = (pool, cdf_ref, cdf_eng, empty)
        elif op == 'sample':
            _, pid, n, ukey, okey = c
            pool, cdf_ref, cdf_eng, empty = pools[pid]
            u = arrays[ukey]
            got = np.asarray(pool.sample(n, u).intarray, np.int64)
            want = arrays[okey]
            stats.samples += n
            bad = got != want
            if bad.any():
                near, tau = sv.boundary_tolerance_mask(cdf_ref, cdf_eng, u)
                # quantisation of the engine's probabilities to its output
                # precision adds to tau for complex64
                stats.sample_mismatch += int(bad.sum())
                outside = bad & ~near
                stats.sample_mismatch_outside_tol += int(outside.sum())
                if outside.any():
                    stats.failures.append('%s: %d sampled indices differ away from CDF '
                                          'boundaries (tau %.2e)' % (where, int(outside.sum()), tau))
        else:
            raise ValueError('unknown trace op %s' % op)
    return stats
