"""Generates the golden fixtures under tests/golden/ by running the reference.

Run in a container that has the reference sources and its CPU runtime built
(`make -C oracle ref`):

    python tests/golden/make_golden.py [--ref /path/to/reference]

What it writes
* gate_matrices.npz — every gate matrix of the reference's Python gate set
  (qgate/simulator/pymatrix.py) at the angles its own matrix tests use
  (tests/test_gate_matrix.py), with and without adjoint.
* traces/<scenario>.json + .npz — boundary traces.  Each scenario is a
  circuit written with the reference's script API and run by the reference's
  own `Simulator` on its C++ CPU runtime in complex128 (the FP64 oracle).  A
  recording wrapper around that runtime logs every call the front-end makes
  across the runtime plugin boundary (the defpkg protocol of
  qgate/simulator/simulator.py:13-23) with its arguments and results:
  probabilities, gathered states, pool probabilities, sampled indices.
  Replaying a trace against another runtime (tests/replay.py) checks it
  against the reference on exactly the calls the reference front-end makes.

The scenarios are synthetic circuits with seeded angles; measurement
outcomes are fixed by seeding numpy's global RNG, which the reference's
executor draws from (qgate/simulator/model_executor.py:117).
"""
import argparse
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.ref_import import reference_root  # noqa: E402


# ------------------------------------------------------------------ recorder

class Log:
    def __init__(self):
        self.calls = []
        self.arrays = {}
        self.next_id = 0

    def new_id(self):
        self.next_id += 1
        return self.next_id

    def arr(self, a):
        key = 'a%d' % len(self.arrays)
        self.arrays[key] = np.array(a)
        return key


def _lt(lane_trans):
    return [[qs.sid, [[int(l.local), int(l.external)] for l in lanes]] for qs, lanes in lane_trans]


def _inner_lt(lane_trans):
    return [(qs.inner, lanes) for qs, lanes in lane_trans]


def _gate(gate_type):
    return [type(gate_type).__name__, [float(a) for a in gate_type.args]]


class RecProcessor:
    def __init__(self, inner, log):
        self.inner, self.log = inner, log

    def synchronize(self):
        self.log.calls.append(['sync'])
        self.inner.synchronize()

    def reset(self):
        self.inner.reset()

    def initialize_qubit_states(self, qs, n_lanes):
        self.log.calls.append(['init', qs.sid, int(n_lanes)])
        self.inner.initialize_qubit_states(qs.inner, n_lanes)

    def reset_qubit_states(self, qs):
        self.log.calls.append(['reset_states', qs.sid])
        self.inner.reset_qubit_states(qs.inner)

    def calc_probability(self, qs, lane):
        p = self.inner.calc_probability(qs.inner, lane)
        self.log.calls.append(['prob', qs.sid, int(lane), float(p)])
        return p

    def join(self, qs, qs_list, n_new):
        self.log.calls.append(['join', qs.sid, [q.sid for q in qs_list], int(n_new)])
        self.inner.join(qs.inner, [q.inner for q in qs_list], n_new)

    def decohere(self, value, prob, qs, lane):
        self.log.calls.append(['decohere', int(value), float(prob), qs.sid, int(lane)])
        return self.inner.decohere(value, prob, qs.inner, lane)

    def decohere_and_separate(self, value, prob, qs0, qs1, qs, lane):
        self.log.calls.append(['separate', int(value), float(prob), qs0.sid, qs1.sid, qs.sid,
                               int(lane)])
        return self.inner.decohere_and_separate(value, prob, qs0.inner, qs1.inner, qs.inner, lane)

    def apply_reset(self, qs, lane):
        self.log.calls.append(['apply_reset', qs.sid, int(lane)])
        self.inner.apply_reset(qs.inner, lane)

    def apply_gate(self, gate_type, adj, qs, lane):
        self.log.calls.append(['gate'] + _gate(gate_type) + [bool(adj), qs.sid, int(lane), []])
        self.inner.apply_gate(gate_type, adj, qs.inner, lane)

    def apply_controlled_gate(self, gate_type, adj, qs, ctrls, target):
        self.log.calls.append(['gate'] + _gate(gate_type) +
                              [bool(adj), qs.sid, int(target), [int(c) for c in ctrls]])
        self.inner.apply_controlled_gate(gate_type, adj, qs.inner, ctrls, target)


class RecStates:
    def __init__(self, inner, sid, processor):
        self.inner, self.sid, self.processor = inner, sid, processor

    def __del__(self):
        # the front-end dropped its last reference (after a join or a
        # separation, qgate/simulator/qubits_handler.py:67-68, :100)
        self.processor.log.calls.append(['delete_states', self.sid])

    def get_n_lanes(self):
        return self.inner.get_n_lanes()

    def reset_lane_states(self):
        self.inner.reset_lane_states()

    def get_lane_state(self, lane):
        return self.inner.get_lane_state(lane)

    def set_lane_state(self, lane, value):
        self.inner.set_lane_state(lane, value)

    def calc_probability(self, lane):
        return self.processor.calc_probability(self, lane)


class RecPool:
    def __init__(self, inner, pid, log):
        self.inner, self.pid, self.log = inner, pid, log

    def sample(self, n_samples, randnum=None):
        if randnum is None:
            randnum = np.random.random_sample([n_samples])
        obs = self.inner.sample(n_samples, randnum)
        self.log.calls.append(['sample', self.pid, int(n_samples), self.log.arr(randnum),
                               self.log.arr(np.asarray(obs.intarray, np.int64))])
        return obs


class RecGetter:
    def __init__(self, inner, gid, log):
        self.inner, self.gid, self.log = inner, gid, log

    def get_states(self, values, offset, mathop, lane_trans, empty_lanes, n_states, start, step):
        # The reference CPU runtime's blocked gather (taken for >= 256 states)
        # evaluates the empty-lane test on the first 256-element block of each
        # thread's span only (qgate/simulator/src/CPUQubitsStatesGetter.cpp:75-83:
        # extSrcIdx is never advanced), so with empty lanes above bit 7 it
        # returns wrong values; its per-element path (< 256 states, :115-116)
        # and the CUDA runtime (qgate/simulator/src/DeviceGetStates.cu:185-189)
        # test every index.  With empty lanes the gather is therefore issued in
        # pieces of fewer than 256 states, which runs the reference's own
        # per-element code.
        if empty_lanes and n_states >= 256:
            for c in range(0, n_states, 255):
                cnt = min(255, n_states - c)
                self.inner.get_states(values, offset + c, mathop, _inner_lt(lane_trans),
                                      empty_lanes, cnt, start + step * c, step)
        else:
            self.inner.get_states(values, offset, mathop, _inner_lt(lane_trans), empty_lanes,
                                  n_states, start, step)
        self.log.calls.append(['get_states', mathop.__name__, _lt(lane_trans),
                               [int(e) for e in empty_lanes], int(n_states), int(start), int(step),
                               int(offset), int(len(values)),
                               self.log.arr(values[offset:offset + n_states])])

    def create_sampling_pool(self, qreg_ordering, n_lanes, n_hidden_lanes, lane_trans,
                             empty_lanes, sampling_pool_factory=None):
        import copy
        lt_before = _lt(lane_trans)
        ordering = [q.id for q in qreg_ordering]
        # The marginal distribution the pool is built on, captured through the
        # reference's own factory hook (qgate/simulator/native_qubits_states_getter.py:50-54).
        captured = {}

        def capture(prob, empty, ordering_):
            captured['prob'] = np.array(prob)
            return None
        lt_copy = [(qs.inner, copy.deepcopy(lanes)) for qs, lanes in lane_trans]
        self.inner.create_sampling_pool(qreg_ordering, n_lanes, n_hidden_lanes, lt_copy,
                                        empty_lanes, capture)
        pid = self.log.new_id()
        self.log.calls.append(['pool', pid, ordering, int(n_lanes), int(n_hidden_lanes), lt_before,
                               [int(e) for e in empty_lanes], sampling_pool_factory is not None,
                               self.log.arr(captured['prob'])])
        if sampling_pool_factory is not None:
            return sampling_pool_factory(captured['prob'], empty_lanes, qreg_ordering)
        inner = self.inner.create_sampling_pool(qreg_ordering, n_lanes, n_hidden_lanes,
                                                _inner_lt(lane_trans), empty_lanes)
        return RecPool(inner, pid, self.log)


class RecRuntime:
    """A defpkg that forwards to the reference's CPU runtime and logs."""

    def __init__(self, inner, log):
        self.inner, self.log = inner, log

    def create_qubit_states(self, dtype):
        qs = self.inner.create_qubit_states(dtype)
        sid = self.log.new_id()
        self.log.calls.append(['new_states', sid])
        return RecStates(qs, sid, RecProcessor(qs.processor, self.log))

    def create_qubits_states_getter(self, dtype):
        g = self.inner.create_qubits_states_getter(dtype)
        gid = self.log.new_id()
        self.log.calls.append(['new_getter', gid])
        return RecGetter(g, gid, self.log)


# ------------------------------------------------------------------ scenarios

def scenarios(qgate):
    from qgate.script import (new_qregs, new_references, new_reference, measure, prob, reset,
                              if_, H, X, Y, Z, S, T, I, SH, Rx, Ry, Rz, U1, U2, U3, ctrl, Swap,
                              Expi, Expii, Expiz)

    def dump_all(sim, qregs, extra=()):
        sim.qubits.set_ordering(list(qregs))
        sim.qubits.states[:]
        sim.qubits.prob[:]
        for q in qregs:
            sim.qubits.calc_probability(q)
        for key in extra:
            sim.qubits.states[key]

    out = {}

    def qft(n, seed):
        rng = np.random.default_rng(seed)
        q = new_qregs(n)
        c = [X(q[i]) for i in range(n) if rng.random() < 0.5]
        for i in range(n):
            c.append(H(q[i]))
            for j in range(i + 1, n):
                c.append(ctrl(q[j]).U1(math.pi / (1 << (j - i)))(q[i]))
        return q, c

    def s_qft(prep):
        q, c = qft(8, 0)
        refs = new_references(len(q))
        c += [prob(refs[i], q[i]) for i in range(len(q))]
        sim = qgate.simulator.cpu(circuit_prep=prep)
        sim.run(c)
        dump_all(sim, q, [slice(3, 200, 7), slice(200, 3, -5), -1, 17])
        pool = sim.qubits.create_sampling_pool(q)
        n = 1 << len(q)
        pool.sample(n, np.linspace(0.5 / n, 1., n, endpoint=False))
        pool.sample(2000, np.random.default_rng(1).random(2000))
        return sim
    out['qft8_one_static'] = lambda: s_qft(qgate.prefs.one_static)
    out['qft8_dynamic'] = lambda: s_qft(qgate.prefs.dynamic)

    def s_random(n, depth, seed):
        rng = np.random.default_rng(seed)
        q = new_qregs(n)
        c = []
        for _ in range(depth):
            ang = rng.uniform(0, 2 * math.pi, (n, 3))
            c += [U3(*ang[i])(q[i]) for i in range(n)]
            perm = rng.permutation(n)
            c += [ctrl(q[perm[2 * k]]).X(q[perm[2 * k + 1]]) for k in range(n // 2)]
        sim = qgate.simulator.cpu(circuit_prep=qgate.prefs.one_static)
        sim.run(c)
        dump_all(sim, q)
        pool = sim.qubits.create_sampling_pool(q)
        pool.sample(5000, np.random.default_rng(seed + 1).random(5000))
        return sim
    out['random_u3cx_10'] = lambda: s_random(10, 5, 10)

    def s_random_dynamic(n, depth, seed):
        """The random U3 + CX circuit under the default dynamic qubit
        grouping: every qubit starts in its own states object, CX gates join
        groups, and measuring every qubit separates them again."""
        rng = np.random.default_rng(seed)
        q = new_qregs(n)
        r = new_references(n)
        c = []
        for _ in range(depth):
            ang = rng.uniform(0, 2 * math.pi, (n, 3))
            c += [U3(*ang[i])(q[i]) for i in range(n)]
            perm = rng.permutation(n)
            c += [ctrl(q[perm[2 * k]]).X(q[perm[2 * k + 1]]) for k in range(n // 2)]
        c += [prob(r[i], q[i]) for i in range(n)]
        c += [measure(r[i], q[i]) for i in rng.permutation(n)]
        sim = qgate.simulator.cpu(circuit_prep=qgate.prefs.dynamic)
        sim.run(c)
        dump_all(sim, q)
        return sim
    out['random_u3cx_12_dynamic'] = lambda: s_random_dynamic(12, 4, 12)
    out['random_u3cx_13'] = lambda: s_random(13, 4, 11)

    def s_gateset():
        q = new_qregs(6)
        c = [H(q[0]), X(q[1]), Y(q[2]), Z(q[3]), S(q[4]), T(q[5]), I(q[0]), SH(q[1]),
             Rx(0.3)(q[2]), Ry(-1.1)(q[3]), Rz(2.2)(q[4]), U1(0.7)(q[5]), U2(0.4, -0.9)(q[0]),
             U3(1.3, 0.2, -0.5)(q[1]), Expii(0.35)(q[2]), Expiz(-0.8)(q[3]),
             S.Adj(q[4]), T.Adj(q[5]), U3(0.9, -0.4, 1.7).Adj(q[2]), SH.Adj(q[3]),
             ctrl(q[0]).H(q[5]), ctrl(q[1], q[2]).Rx(0.6)(q[4]), ctrl(q[3]).U3(0.1, 0.2, 0.3)(q[0]),
             ctrl(q[5], q[4], q[3]).Y(q[1]), ctrl(q[2]).Z(q[0]), ctrl(q[4]).T.Adj(q[3]),
             Swap(q[0], q[5]), Swap(q[1], q[3]),
             Expi(0.45)(X(q[0]), Y(q[2]), Z(q[4])), Expi(-0.2)(Z(q[1]), Z(q[5]))]
        sim = qgate.simulator.cpu(circuit_prep=qgate.prefs.one_static)
        sim.run(c)
        dump_all(sim, q)
        return sim
    out['gateset6'] = s_gateset

    def s_multicontrol():
        sims = []
        for n in (3, 5, 9):
            q = new_qregs(n)
            c = [H(x) for x in q[:-1]] + [ctrl(q[:-1]).X(q[-1])] + [ctrl(q[0], q[-1]).Ry(0.7)(q[1])]
            sim = qgate.simulator.cpu(circuit_prep=qgate.prefs.dynamic)
            sim.run(c)
            dump_all(sim, q)
            sims.append(sim)
        return sims
    out['multicontrol'] = s_multicontrol

    def s_pauli():
        q = new_qregs(5)
        rng = np.random.default_rng(5)
        c = [U3(*rng.uniform(0, 2 * math.pi, 3))(x) for x in q]
        c += [ctrl(q[0]).X(q[1]), ctrl(q[2]).X(q[3]), ctrl(q[4]).X(q[0])]
        refs = new_references(6)
        c += [prob(refs[0], [Z(q[0])]), prob(refs[1], [X(q[1])]), prob(refs[2], [Y(q[2])]),
              prob(refs[3], [X(q[0]), Y(q[1]), Z(q[3])]), prob(refs[4], [Z(q[2]), Z(q[4])]),
              prob(refs[5], [Y(q[0]), X(q[4]), X(q[3]), Z(q[1])])]
        sim = qgate.simulator.cpu(circuit_prep=qgate.prefs.one_static)
        sim.run(c)
        dump_all(sim, q)
        return sim
    out['pauli_prob5'] = s_pauli

    def s_measure(prep, seed):
        np.random.seed(seed)
        q = new_qregs(6)
        r = new_references(6)
        c = [H(q[0]), ctrl(q[0]).X(q[1]), Ry(1.1)(q[2]), ctrl(q[2]).H(q[3]), Rx(0.4)(q[4]),
             measure(r[0], q[0]), measure(r[2], q[2]), reset(q[2])]
        # if_ after a measure only works with dynamic preprocessing in the
        # reference (static preps hit an AttributeError in
        # qgate/simulator/model_executor.py:76).
        c += [if_(r[0], 1, [X(q[5])])] if prep == qgate.prefs.dynamic else [X(q[5])]
        c += [ctrl(q[1]).Rz(0.3)(q[4]), measure(r[4], q[4]),
             reset(q[4]), H(q[4]), ctrl(q[4]).X(q[3]), measure(r[3], [X(q[3]), Z(q[1])]),
             measure(r[5], q[5]), reset(q[5])]
        sim = qgate.simulator.cpu(circuit_prep=prep)
        sim.run(c)
        dump_all(sim, q)
        return sim
    out['measure_reset_if_dynamic'] = lambda: s_measure(qgate.prefs.dynamic, 3)
    out['measure_reset_if_static'] = lambda: s_measure(qgate.prefs.static, 4)
    out['measure_reset_if_onestatic'] = lambda: s_measure(qgate.prefs.one_static, 5)

    def s_join():
        q = new_qregs(9)
        rng = np.random.default_rng(7)
        c = [Ry(a)(x) for a, x in zip(rng.uniform(-3, 3, 9), q)]
        c += [ctrl(q[0]).X(q[1]), ctrl(q[2]).X(q[3]), ctrl(q[4]).X(q[5]), ctrl(q[1]).X(q[2]),
              ctrl(q[6], q[7]).X(q[8]), ctrl(q[3]).Rz(0.4)(q[6]), ctrl(q[5]).X(q[8])]
        sim = qgate.simulator.cpu(circuit_prep=qgate.prefs.dynamic)
        sim.run(c)
        dump_all(sim, q)
        return sim
    out['join9_dynamic'] = s_join

    def s_pools():
        q = new_qregs(10)
        c = [H(x) for x in q[::2]] + [X(x) for x in q[1::2]] + [ctrl(q[0]).Ry(0.9)(q[3]),
                                                                   Rx(0.3)(q[6])]
        sim = qgate.simulator.cpu(circuit_prep=qgate.prefs.one_static)
        sim.run(c)
        dump_all(sim, q)
        extra = new_qregs(3)

        class Dummy:
            def __init__(self, prob, empty_lanes, qreg_ordering):
                self.prob = prob
        sim.qubits.create_sampling_pool(q[::2], Dummy)            # hidden lanes
        sim.qubits.create_sampling_pool([q[7], q[2], q[5]], Dummy)  # hidden, permuted
        p1 = sim.qubits.create_sampling_pool(q[1::2] + [q[0]])    # hidden lanes, sampled
        p1.sample(3000, np.random.default_rng(2).random(3000))
        ordering = [extra[0], q[3], q[0], extra[1], q[6], extra[2], q[9]]
        p2 = sim.qubits.create_sampling_pool(ordering)            # empty + hidden lanes
        p2.sample(3000, np.random.default_rng(3).random(3000))
        sim.qubits.set_ordering([extra[0]] + list(q) + [extra[1]])  # empty lanes in states
        sim.qubits.states[:]
        sim.qubits.prob[::-3]
        return sim
    out['pools10'] = s_pools

    def s_big():
        q, c = qft(14, 9)
        sim = qgate.simulator.cpu(circuit_prep=qgate.prefs.one_static)
        sim.run(c)
        sim.qubits.set_ordering(list(q))
        sim.qubits.prob[:]
        for x in q[::3]:
            sim.qubits.calc_probability(x)
        pool = sim.qubits.create_sampling_pool(q)
        pool.sample(10000, np.random.default_rng(4).random(10000))
        return sim
    out['qft14'] = s_big
    return out


GATE_ANGLES = [0., math.pi / 4., -math.pi / 4., math.pi / 2., -math.pi / 2., math.pi, -math.pi,
               2. * math.pi, 0.3, -1.7]


def gate_matrices(qgate):
    import qgate.model.gate_type as gtype
    import qgate.simulator.pymatrix  # noqa: F401  (attaches pymat)
    rows = {}
    names0 = ['ID', 'X', 'Y', 'Z', 'H', 'S', 'T', 'SH']
    names1 = ['U1', 'RX', 'RY', 'RZ', 'ExpiI', 'ExpiZ']
    for nm in names0:
        g = getattr(gtype, nm)()
        rows['%s||0' % nm] = g.pymat()
    for nm in names1:
        for a in GATE_ANGLES:
            rows['%s|%r|0' % (nm, a)] = getattr(gtype, nm)(a).pymat()
    for a in GATE_ANGLES:
        for b in GATE_ANGLES[::3]:
            rows['U2|%r,%r|0' % (a, b)] = gtype.U2(a, b).pymat()
            for c in GATE_ANGLES[::4]:
                rows['U|%r,%r,%r|0' % (a, b, c)] = gtype.U(a, b, c).pymat()
    return rows


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', default=reference_root())
    args = ap.parse_args()
    from oracle.ref_import import import_reference
    qgate = import_reference(args.ref)
    import qgate.simulator.cpuruntime as cpuruntime
    from qgate.simulator.simulator import Simulator

    mats = gate_matrices(qgate)
    np.savez_compressed(os.path.join(HERE, 'gate_matrices.npz'),
                        keys=np.array(list(mats.keys())),
                        mats=np.array(list(mats.values()), np.complex128))

    tdir = os.path.join(HERE, 'traces')
    os.makedirs(tdir, exist_ok=True)
    for name, fn in scenarios(qgate).items():
        log = Log()
        rec = RecRuntime(cpuruntime, log)
        orig_cpu = qgate.simulator.cpu
        qgate.simulator.cpu = lambda **prefs: Simulator(rec, **prefs)
        try:
            np.random.seed(1234)
            fn()
        finally:
            qgate.simulator.cpu = orig_cpu
        with open(os.path.join(tdir, name + '.json'), 'w') as f:
            json.dump({'scenario': name, 'dtype': 'float64', 'calls': log.calls}, f)
        np.savez_compressed(os.path.join(tdir, name + '.npz'), **log.arrays)
        print('%-28s %5d calls %4d arrays' % (name, len(log.calls), len(log.arrays)))


if __name__ == '__main__':
    main()
