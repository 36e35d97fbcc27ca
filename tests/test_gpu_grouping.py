"""GPU tests of the qubit-grouping policy: lazy joins (a product of the
sources' buffers, formed when first read), separations left as views of the
source (formed in place once the source is gone), lazy |0...0> allocation,
and copy-on-write of a buffer that a lazy object still reads.  Results are
checked against the oracle (complex128 numpy) or the reference's recorded
trace; the counters (qg_grouping_stats) show the kron passes, allocations
and copies the policy saved."""
import numpy as np
import pytest

from oracle import statevec as sv
from tests import replay
from tests.gpu_helpers import apply_ops, new_state, random_ops

pytestmark = pytest.mark.gpu

ATOL = {np.float64: 1e-12, np.float32: 2e-6}
DTYPES = [np.float64, np.float32]
IDS = ['c128', 'c64']


def _stats(reset=True):
    from qgate_gb300 import _native as nat
    return nat.grouping_stats(reset=reset)


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_dynamic_prep_trace_forms_each_state_once(rt, dtype):
    """The reference front-end's dynamic qubit grouping on a 12-qubit random
    U3 + CX circuit (recorded trace: 45 states objects, 11 joins, 11
    separations; every dropped object deleted as the front-end dropped it):
    same results as the reference, no kron pass (every joined factor is
    still |0> with its gates pending), one 12-lane buffer, and every
    separation formed in place in that buffer."""
    calls, arrays = replay.load_trace('random_u3cx_12_dynamic')
    _stats()
    stats = replay.replay(calls, arrays, rt, dtype)
    assert not stats.failures, stats.failures[:5]
    g = _stats()
    n_init = sum(1 for c in calls if c[0] == 'init')
    assert g['joins'] == 11 and g['separates'] == 11, g
    assert g['krons'] == 0, g
    assert g['inplace'] == 11 and g['copies'] == 0 and g['cow'] == 0, g
    # one 12-lane buffer plus the 1-lane states of the measured qubits,
    # against one buffer per initialize call (45) when every object allocates
    assert g['allocs'] <= 13 < n_init, (g, n_init)


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_join_chain_with_an_observation_between(rt, dtype):
    """22 one-qubit groups joined pairwise, then into one state, like the
    front-end's dynamic grouping of a C1-style layer of U3 + CX; one
    probability read between the joins forms that group alone.  The final
    state matches the oracle; the chain costs one kron pass (the observed
    group's buffer with the still-|0> rest) instead of one per join."""
    rng = np.random.default_rng(41)
    n = 22
    _stats()
    singles, ops_of = [], []
    for q in range(n):
        qs = new_state(rt, 1, dtype)
        ops = [('g', 'U', tuple(rng.uniform(0, 3, 3)), False, 0, ())]
        apply_ops(qs, ops)
        singles.append(qs)
        ops_of.append(ops)
    # pairs: group k holds qubits 2k (lane 1) and 2k + 1 (lane 0)
    pairs, pair_ops = [], []
    for k in range(n // 2):
        qs = rt.create_qubit_states(dtype)
        qs.processor.initialize_qubit_states(qs, 2)
        qs.processor.join(qs, [singles[2 * k], singles[2 * k + 1]], 0)
        ops = [('g', nm, a, adj, t + 1, c) for _, nm, a, adj, t, c in ops_of[2 * k]]
        ops += [('g', nm, a, adj, t, c) for _, nm, a, adj, t, c in ops_of[2 * k + 1]]
        cx = [('g', 'X', (), False, 0, (1,))]
        apply_ops(qs, cx)
        pairs.append(qs)
        pair_ops.append(ops + cx)
    # observe group 3 before the final join: it is formed on its own
    p3 = pairs[3].processor.calc_probability(pairs[3], 0)
    psi3 = sv.run_ops(2, pair_ops[3])
    assert abs(p3 - sv.calc_probability(psi3, 0)) < ATOL[dtype]
    for qs in singles:
        qs.delete()
    full = rt.create_qubit_states(dtype)
    full.processor.initialize_qubit_states(full, n)
    full.processor.join(full, pairs, 0)
    # pairs[0] at the highest lanes: pair k at lanes 2 (n/2 - 1 - k) ..
    ops_full = []
    for k, ops in enumerate(pair_ops):
        off = 2 * (n // 2 - 1 - k)
        ops_full += [('g', nm, a, adj, t + off, tuple(c + off for c in cs))
                     for _, nm, a, adj, t, cs in ops]
    layer = [('g', 'X', (), False, q + 1, (q,)) for q in range(0, n - 1, 2)]
    apply_ops(full, layer)
    psi = sv.run_ops(n, ops_full + layer)
    for lane in (0, 7, n - 1):
        got = full.processor.calc_probability(full, lane)
        assert abs(got - sv.calc_probability(psi, lane)) < 4 * ATOL[dtype], lane
    for qs in pairs:
        qs.delete()
    g = _stats()
    assert g['joins'] == n // 2 + 1, g
    assert g['krons'] == 1, g
    # the observed pair's buffer and the joined state's
    assert g['allocs'] == 2, g
    full.delete()


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_join_sources_stay_usable_copy_on_write(rt, dtype):
    """After a join the sources keep their amplitudes: a gate applied to a
    source (whose buffer the lazy product still reads) copies the buffer
    first, so the product still holds the source as it was at the join."""
    rng = np.random.default_rng(42)
    a_ops, b_ops = random_ops(rng, 4, 20), random_ops(rng, 3, 15)
    a, b = new_state(rt, 4, dtype), new_state(rt, 3, dtype)
    apply_ops(a, a_ops)
    apply_ops(b, b_ops)
    a.processor.synchronize()  # a and b formed and their gates run
    _stats()
    joined = rt.create_qubit_states(dtype)
    joined.processor.initialize_qubit_states(joined, 9)
    joined.processor.join(joined, [a, b], 2)
    x = [('g', 'X', (), False, 0, ())]
    apply_ops(a, x)
    psi_a = sv.run_ops(4, a_ops)
    psi_b = sv.run_ops(3, b_ops)
    assert np.allclose(a.get_raw(), sv.run_ops(4, x, psi=psi_a.copy()), atol=4 * ATOL[dtype])
    want = sv.join([psi_a, psi_b], 2)
    assert np.allclose(joined.get_raw(), want, atol=4 * ATOL[dtype])
    g = _stats()
    assert g['cow'] == 1 and g['krons'] == 1, g
    for qs in (a, b, joined):
        qs.delete()


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
@pytest.mark.parametrize('keep_source', [False, True], ids=['source_deleted', 'source_kept'])
def test_separation_in_place_or_copy(rt, dtype, keep_source):
    """decohere_and_separate on a 16-lane state at every fourth lane, both
    outcomes: the remaining lanes are formed in place when the source was
    deleted first, by copy when the source is still alive (and the source
    keeps its amplitudes)."""
    rng = np.random.default_rng(43)
    n = 16
    for lane in (0, 5, 10, 15):
        for value in (0, 1):
            ops = [('g', 'H', (), False, q, ()) for q in range(n)] + random_ops(rng, n, 40)
            psi = sv.run_ops(n, ops)
            p = sv.calc_probability(psi, lane)
            if (p if value == 0 else 1. - p) < 1e-3:
                continue  # an outcome the state (nearly) never gives
            qs = new_state(rt, n, dtype)
            apply_ops(qs, ops)
            qs0, qs1 = rt.create_qubit_states(dtype), rt.create_qubit_states(dtype)
            qs.processor.initialize_qubit_states(qs0, n - 1)
            qs.processor.initialize_qubit_states(qs1, 1)
            _stats()
            qs.processor.decohere_and_separate(value, p, qs0, qs1, qs, lane)
            before = qs.get_raw() if keep_source else None
            if not keep_source:
                qs.delete()
            w0, w1 = sv.decohere_and_separate(psi, value, p, lane)
            assert np.allclose(qs0.get_raw(), w0, atol=4 * ATOL[dtype]), (lane, value)
            assert np.array_equal(qs1.get_raw(), w1.astype(qs1.get_raw().dtype)), (lane, value)
            g = _stats()
            if keep_source:
                assert g['copies'] == 1 and g['inplace'] == 0, g
                assert np.array_equal(qs.get_raw(), before)
                qs.delete()
            else:
                assert g['inplace'] == 1 and g['copies'] == 0, g
            qs0.delete()
            qs1.delete()


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_separate_then_gates_and_rejoin(rt, dtype):
    """Gates queued on a separated view, then the view joined with the
    measured qubit again: the view is formed (in place) before the join
    reads it; against the oracle."""
    rng = np.random.default_rng(44)
    n = 10
    ops = [('g', 'H', (), False, q, ()) for q in range(n)] + random_ops(rng, n, 40)
    qs = new_state(rt, n, dtype)
    apply_ops(qs, ops)
    psi = sv.run_ops(n, ops)
    lane, value = 4, 1
    p = sv.calc_probability(psi, lane)
    qs0, qs1 = rt.create_qubit_states(dtype), rt.create_qubit_states(dtype)
    qs.processor.initialize_qubit_states(qs0, n - 1)
    qs.processor.initialize_qubit_states(qs1, 1)
    qs.processor.decohere_and_separate(value, p, qs0, qs1, qs, lane)
    qs.delete()
    more = random_ops(rng, n - 1, 20)
    apply_ops(qs0, more)
    w0, w1 = sv.decohere_and_separate(psi, value, p, lane)
    w0 = sv.run_ops(n - 1, more, psi=w0)
    joined = rt.create_qubit_states(dtype)
    joined.processor.initialize_qubit_states(joined, n)
    joined.processor.join(joined, [qs1, qs0], 0)
    want = sv.join([w1, w0], 0)
    assert np.allclose(joined.get_raw(), want, atol=4 * ATOL[dtype])
    for x in (qs0, qs1, joined):
        x.delete()


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_lazy_products_read_by_getter_pool_and_compiled_runs(rt, dtype):
    """Joined objects that were never read (products of buffers and |0>
    factors with gates pending) go straight into a gather with swapped lanes,
    a sampling pool and a compiled-circuit run; each matches the oracle."""
    from qgate_gb300.circuit import Lane, abs2, gate_type
    from qgate_gb300.compiled import CompiledCircuit
    rng = np.random.default_rng(45)
    parts, psis = [], []
    for k in (3, 2, 4):
        qs = new_state(rt, k, dtype)
        ops = random_ops(rng, k, 12)
        apply_ops(qs, ops)
        parts.append(qs)
        psis.append(sv.run_ops(k, ops))
    parts[0].processor.synchronize()  # the first part formed, the others not
    a = rt.create_qubit_states(dtype)
    a.processor.initialize_qubit_states(a, 5)
    a.processor.join(a, [parts[0], parts[1]], 0)
    b = rt.create_qubit_states(dtype)
    b.processor.initialize_qubit_states(b, 6)
    b.processor.join(b, [parts[2]], 2)
    psi_a = sv.join([psis[0], psis[1]], 0)
    psi_b = sv.join([psis[2]], 2)
    # gather: lanes of a and b interleaved in the external order
    la = [Lane(l, e) for l, e in zip(range(5), (0, 2, 4, 6, 8))]
    lb = [Lane(l, e) for l, e in zip(range(6), (1, 3, 5, 7, 9, 10))]
    getter = rt.create_qubits_states_getter(dtype)
    probs = np.empty(1 << 11, dtype)
    getter.get_states(probs, 0, abs2, [(a, la), (b, lb)], [], 1 << 11, 0, 1)
    pa, pb = np.abs(psi_a) ** 2, np.abs(psi_b) ** 2
    want = np.zeros(1 << 11)
    for x in range(1 << 11):
        ia = sum(((x >> e) & 1) << l for l, e in zip(range(5), (0, 2, 4, 6, 8)))
        ib = sum(((x >> e) & 1) << l for l, e in zip(range(6), (1, 3, 5, 7, 9, 10)))
        want[x] = pa[ia] * pb[ib]
    assert np.allclose(probs, want, atol=4 * ATOL[dtype])
    # a pool over b alone, then a compiled run on a fresh lazy product
    pool = getter.create_sampling_pool(list(range(6)), 6, 0, [(b, [Lane(l, l) for l in range(6)])],
                                       [])
    u = rng.random(2000)
    obs = np.asarray(pool.sample(len(u), u).intarray)
    assert np.mean(obs == sv.SamplingPool(pb).sample(u)) > 0.99
    pool.delete()
    c = rt.create_qubit_states(dtype)
    c.processor.initialize_qubit_states(c, 7)
    c.processor.join(c, [parts[1]], 5)
    cops = random_ops(rng, 7, 16, max_controls=1)
    circ = CompiledCircuit(dtype, [(gate_type(nm, *args), adj, t, list(cs))
                                   for _, nm, args, adj, t, cs in cops], graph=True)
    circ.run(c)
    want_c = sv.run_ops(7, cops, psi=sv.join([psis[1]], 5))
    assert np.allclose(c.get_raw(), want_c, atol=4 * ATOL[dtype])
    for x in parts + [a, b, c]:
        x.delete()


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_x_gates_on_a_basis_state_fold_into_it(rt, dtype):
    """X gates (with or without controls) that reach a reset state before any
    other gate on their lanes are applied to its basis value: a circuit of
    such gates alone takes no pass and gives the exact basis state; mixed
    with other gates (an X after an H on its lane, an X whose control saw an
    earlier gate, controls at 0 and at 1, an adjoint X) and after a reset of
    a live state, the result still matches the oracle."""
    from qgate_gb300 import _native as nat
    n = 9
    flips = [('g', 'X', (), False, 3, ()), ('g', 'X', (), False, 5, (3,)),
             ('g', 'X', (), True, 1, (3, 5)), ('g', 'X', (), False, 7, (6,)),
             ('g', 'X', (), False, 8, (6, 3))]
    want = sv.run_ops(n, flips)
    assert abs(want[(1 << 1) | (1 << 3) | (1 << 5)]) == 1.
    qs = new_state(rt, n, dtype)
    nat.gate_stats(reset=True)
    apply_ops(qs, flips)
    got = qs.get_raw()
    assert nat.gate_stats(reset=True)['passes'] == 0
    assert np.array_equal(got, want.astype(got.dtype))
    rng = np.random.default_rng(46)
    mixed = ([('g', 'H', (), False, 0, ()), ('g', 'X', (), False, 0, ()),
              ('g', 'X', (), False, 2, (0,)), ('g', 'X', (), False, 4, ())] + flips +
             random_ops(rng, n, 30) + [('g', 'X', (), False, 6, ())])
    qs2 = new_state(rt, n, dtype)
    apply_ops(qs2, mixed)
    assert np.allclose(qs2.get_raw(), sv.run_ops(n, mixed), atol=4 * ATOL[dtype])
    qs2.processor.reset_qubit_states(qs2)
    nat.gate_stats(reset=True)
    apply_ops(qs2, flips + mixed)
    assert np.allclose(qs2.get_raw(), sv.run_ops(n, flips + mixed), atol=4 * ATOL[dtype])
    assert nat.gate_stats(reset=True)['passes'] > 0
    for x in (qs, qs2):
        x.delete()
