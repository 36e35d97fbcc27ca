"""Oracle runtime: the numpy restatement (`oracle.statevec`) behind the same
runtime plugin protocol as the GB300 runtime and the reference's runtimes
(qgate/simulator/pyruntime.py:10-328, qgate/simulator/native_*.py).

TEST INFRASTRUCTURE ONLY — part of the oracle, never part of the product.  Used by the
CPU tests to replay the reference's boundary traces (pinning the oracle to
the reference's own outputs) and to produce expected values for GPU tests.
"""
import numpy as np

from . import statevec as sv


class SampleList:
    def __init__(self, values):
        self.intarray = values


class OracleProcessor:
    def __init__(self, dtype):
        self.dtype = dtype

    def synchronize(self):
        pass

    def reset(self):
        pass

    def initialize_qubit_states(self, qs, n_lanes):
        qs.psi = np.zeros(1 << n_lanes, qs.cdtype)
        qs.reset_lane_states()

    def reset_qubit_states(self, qs):
        qs.psi[:] = 0.
        qs.psi[0] = 1.
        qs.reset_lane_states()

    def calc_probability(self, qs, lane):
        return sv.calc_probability(qs.psi, lane)

    def join(self, qs, qs_list, n_new):
        qs.psi[:] = sv.join([q.psi for q in qs_list], n_new)

    def decohere(self, value, prob, qs, lane):
        sv.decohere(qs.psi, value, prob, lane)
        return value

    def decohere_and_separate(self, value, prob, qs0, qs1, qs, lane):
        p0, p1 = sv.decohere_and_separate(qs.psi, value, prob, lane)
        qs0.psi[:] = p0
        qs1.psi[:] = p1
        return value

    def apply_reset(self, qs, lane):
        sv.apply_reset(qs.psi, lane)

    def _mat(self, gate_type, adjoint):
        return sv.gate_matrix(type(gate_type).__name__, tuple(gate_type.args), adjoint)

    def apply_gate(self, gate_type, adjoint, qs, lane):
        sv.apply_gate(qs.psi, self._mat(gate_type, adjoint), lane)

    def apply_controlled_gate(self, gate_type, adjoint, qs, ctrls, target):
        sv.apply_controlled_gate(qs.psi, self._mat(gate_type, adjoint), list(ctrls), target)


class OracleQubitStates:
    def __init__(self, dtype):
        self.processor = OracleProcessor(dtype)
        self.cdtype = np.complex128 if dtype == np.float64 else np.complex64
        self.psi = None

    def get_n_lanes(self):
        return int(self.psi.size).bit_length() - 1

    def reset_lane_states(self):
        self.lane_states = [-1] * self.get_n_lanes()

    def get_lane_state(self, lane):
        return self.lane_states[lane]

    def set_lane_state(self, lane, value):
        self.lane_states[lane] = value

    def calc_probability(self, lane):
        return self.processor.calc_probability(self, lane)


def _tables(lane_trans):
    out = []
    for qs, lanes in lane_trans:
        table = [None] * len(lanes)
        for lane in lanes:
            table[lane.local] = lane.external
        out.append((qs.psi, table))
    return out


class OraclePool:
    def __init__(self, prob, empty_lanes):
        self.pool = sv.SamplingPool(prob, empty_lanes)

    def sample(self, n_samples, randnum=None):
        if randnum is None:
            randnum = np.random.random_sample([n_samples])
        return SampleList(self.pool.sample(np.asarray(randnum)[:n_samples]))


class OracleGetter:
    def __init__(self, dtype):
        self.dtype = dtype

    def get_states(self, values, offset, mathop, lane_trans, empty_lanes, n_states, start, step):
        mask = 0
        for e in empty_lanes:
            mask |= 1 << e
        if not lane_trans:
            values[offset:offset + n_states] = 0.
            if start == 0:
                values[offset] = 1.
            return
        v = sv.get_states(_tables(lane_trans), mathop.__name__, n_states, start, step, mask,
                          dtype=values.dtype)
        values[offset:offset + n_states] = v

    def create_sampling_pool(self, qreg_ordering, n_lanes, n_hidden_lanes, lane_trans,
                             empty_lanes, sampling_pool_factory=None):
        hidden = n_lanes
        for qs, lanes in lane_trans:
            for lane in lanes:
                if lane.external == -1:
                    lane.external = hidden
                    hidden += 1
        prob = sv.marginal_probabilities(_tables(lane_trans), n_lanes, n_hidden_lanes)
        if sampling_pool_factory is not None:
            return sampling_pool_factory(prob.astype(self.dtype), empty_lanes, qreg_ordering)
        return OraclePool(prob, empty_lanes)


def create_qubit_states(dtype):
    return OracleQubitStates(dtype)


def create_qubits_states_getter(dtype):
    return OracleGetter(dtype)
