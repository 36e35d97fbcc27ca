"""GPU parity of the lane-permuted gather, the marginal probability array and
the FP64 sampling pool against the oracle, plus the reference's own
known-answer sampling tests (tests/test_sampling_pool.py in the reference:
midpoint uniforms on the uniform state give the identity indices; empty lanes
read 0; hidden lanes are summed out)."""
import numpy as np
import pytest

from oracle import statevec as sv
from tests.gpu_helpers import ATOL, Lane, abs2, apply_ops, new_state, null, random_ops
from tests.pool_model import fixed_point_samples

pytestmark = pytest.mark.gpu

DTYPES = [np.float64, np.float32]
IDS = ['c128', 'c64']


def _build(rt, dtype, sizes, seed):
    rng = np.random.default_rng(seed)
    states, psis = [], []
    for k in sizes:
        ops = random_ops(rng, k, 15)
        qs = new_state(rt, k, dtype)
        apply_ops(qs, ops)
        states.append(qs)
        psis.append(sv.run_ops(k, ops, np.complex128))
    return rng, states, psis


def _lane_trans(states, tables):
    return [(qs, [Lane(l, e) for l, e in enumerate(t)]) for qs, t in zip(states, tables)]


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_get_states_permuted_empty_slices(rt, dtype):
    sizes = [3, 2, 4]
    rng, states, psis = _build(rt, dtype, sizes, 11)
    n_lanes = sum(sizes)
    empty = [1, 7]
    n_qregs = n_lanes + len(empty)
    ext = [e for e in rng.permutation(n_qregs) if e not in empty]
    tables, i = [], 0
    for k in sizes:
        tables.append([int(e) for e in ext[i:i + k]])
        i += k
    mask = (1 << 1) | (1 << 7)
    N = 1 << n_qregs
    getter = rt.create_qubits_states_getter(dtype)
    for mathop, name in ((null, 'null'), (abs2, 'abs2')):
        for start, step, count in ((0, 1, N), (5, 3, (N - 5 + 2) // 3), (N - 1, -1, N),
                                   (N - 2, -7, 100), (17, 1, 1)):
            vd = (np.complex128 if dtype == np.float64 else np.complex64) if name == 'null' \
                else dtype
            values = np.zeros(count + 3, vd)
            getter.get_states(values, 3, mathop, _lane_trans(states, tables), empty, count, start,
                              step)
            want = sv.get_states(list(zip(psis, tables)), name, count, start, step, mask)
            assert np.allclose(values[3:], want, atol=ATOL[dtype] * 2), (name, start, step)


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_get_states_identity_ranges(rt, dtype):
    """One state read in its own lane order (the streaming gather): whole
    state, ranges with odd starts and lengths, single items, and outputs at
    odd offsets of the caller's array."""
    rng, states, psis = _build(rt, dtype, [9], 4)
    qs, psi = states[0], psis[0]
    N = 1 << 9
    getter = rt.create_qubits_states_getter(dtype)
    ident = [(qs, [Lane(l, l) for l in range(9)])]
    for mathop, name in ((null, 'null'), (abs2, 'abs2')):
        vd = (np.complex128 if dtype == np.float64 else np.complex64) if name == 'null' else dtype
        for start, count in ((0, N), (1, N - 1), (3, 257), (N - 1, 1), (128, 7), (0, 5)):
            for off in (0, 1, 3):
                values = np.zeros(count + off, vd)
                getter.get_states(values, off, mathop, ident, [], count, start, 1)
                want = sv.get_states([(psi, list(range(9)))], name, count, start, 1, 0)
                assert np.allclose(values[off:], want, atol=ATOL[dtype] * 2), (name, start, off)


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_get_states_range_errors(rt, dtype):
    _, states, _ = _build(rt, dtype, [3], 12)
    getter = rt.create_qubits_states_getter(dtype)
    values = np.zeros(16, dtype)
    lt = _lane_trans(states, [[0, 1, 2]])
    with pytest.raises(ValueError):
        getter.get_states(values, 0, abs2, lt, [], 4, 6, 1)   # end beyond 2^3
    with pytest.raises(ValueError):
        getter.get_states(values, 0, abs2, _lane_trans(states, [[0, 1, 2]]), [], 2, 8, 1)


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_marginal_probabilities_hidden_lanes(rt, dtype):
    """Pool over a permuted subset of lanes of two states; the other lanes
    are hidden and summed out (placed above the pool lanes, in order of
    appearance, as the runtime does)."""
    sizes = [5, 4]
    rng, states, psis = _build(rt, dtype, sizes, 13)
    n_total = sum(sizes)
    getter = rt.create_qubits_states_getter(dtype)
    for n_pool in (1, 3, 6, 9):
        chosen = rng.permutation(n_total)[:n_pool]   # global lane -> pool position
        pos = {int(g): j for j, g in enumerate(chosen)}
        tables, g = [], 0
        for k in sizes:
            tables.append([pos.get(g + q, -1) for q in range(k)])
            g += k
        captured = {}

        def factory(prob, empty_lanes, ordering):
            captured['p'] = prob
        getter.create_sampling_pool(list(range(n_pool)), n_pool, n_total - n_pool,
                                    _lane_trans(states, tables), [], factory)
        h, otables = n_pool, []
        for t in tables:
            row = []
            for e in t:
                if e == -1:
                    row.append(h)
                    h += 1
                else:
                    row.append(e)
            otables.append(row)
        want = sv.marginal_probabilities(list(zip(psis, otables)), n_pool, n_total - n_pool)
        assert captured['p'].dtype == dtype
        assert np.allclose(captured['p'], want, atol=ATOL[dtype] * 2), n_pool


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_sampling_pool_midpoints_identity_24q(rt, dtype):
    """The reference's golden-vector test at its CUDA size (24 qubits):
    H on every qubit, uniforms at bin midpoints (k + 1/2)/2^n -> index k."""
    n = 24
    qs = new_state(rt, n, dtype)
    apply_ops(qs, [('g', 'H', (), False, q, ()) for q in range(n)])
    getter = rt.create_qubits_states_getter(dtype)
    lt = _lane_trans([qs], [list(range(n))])
    pool = getter.create_sampling_pool(list(range(n)), n, 0, lt, [])
    N = 1 << n
    u = (np.arange(N, dtype=np.float64) + 0.5) / N
    obs = pool.sample(N, u)
    assert np.array_equal(np.asarray(obs.intarray), np.arange(N))


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_sampling_pool_empty_lanes_and_random(rt, dtype):
    sizes = [6]
    rng, states, psis = _build(rt, dtype, sizes, 14)
    getter = rt.create_qubits_states_getter(dtype)
    empty = [0, 4, 8]
    # pool lanes are numbered 0..5; zero bits for the empty lanes are inserted
    # into each sampled index
    lt = _lane_trans(states, [list(range(6))])
    pool = getter.create_sampling_pool(list(range(9)), 6, 0, lt, empty)
    u = rng.random(20000)
    got = np.asarray(pool.sample(len(u), u).intarray)
    prob = sv.marginal_probabilities(list(zip(psis, [list(range(6))])), 6, 0)
    want = sv.SamplingPool(prob, empty).sample(u)
    bad = got != want
    if bad.any():
        cdf_ref = np.cumsum(prob) / prob.sum()
        # only uniforms within float rounding of a boundary may differ
        assert np.all(np.abs(u[bad][:, None] - cdf_ref[None, :]).min(axis=1) < 1e-6)
    assert np.all((got & ((1 << 0) | (1 << 4) | (1 << 8))) == 0)


EDGE_U = [0.0, -0.0, 1.0, 1.5, -0.5, float('nan'), 5e-324, 1. - 2. ** -53, 0.5]


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_sampling_pool_fixed_point_exact(rt, dtype):
    """Samples equal, bit for bit, the integer model of the pool's CDF built
    from the engine's own probabilities, both for a pool read straight from
    the state (lanes in order) and for one built from the marginal (lanes
    reversed); and they agree with the oracle's FP64 pool except within
    rounding of a CDF boundary."""
    n = 14
    rng, states, psis = _build(rt, dtype, [n], 21)
    qs, psi = states[0], psis[0]
    getter = rt.create_qubits_states_getter(dtype)
    u = np.concatenate([rng.random(100000), EDGE_U])
    for table in (list(range(n)), list(range(n))[::-1]):
        lanes = [(qs, [Lane(l, e) for l, e in enumerate(table)])]
        probs = np.empty(1 << n, dtype)
        getter.get_states(probs, 0, abs2, lanes, [], 1 << n, 0, 1)
        pool = getter.create_sampling_pool(list(range(n)), n, 0, lanes, [])
        got = np.asarray(pool.sample(len(u), u).intarray)
        pool.delete()
        assert np.array_equal(got, fixed_point_samples(probs, u)), table[:2]
        prob_ref = sv.marginal_probabilities([(psi, table)], n, 0)
        want = sv.SamplingPool(prob_ref).sample(u[:100000])
        cdf_ref = np.cumsum(prob_ref) / prob_ref.sum()
        cdf_eng = np.cumsum(probs.astype(np.float64))
        near, tau = sv.boundary_tolerance_mask(cdf_ref, cdf_eng / cdf_eng[-1], u[:100000])
        assert np.array_equal(got[:100000][~near], want[~near]), tau
        assert np.mean(near) < 0.01, tau


def test_sampling_pool_fixed_point_exact_25q(rt):
    """A 25-qubit complex64 pool: 8192 tiles of 4096, so the prefix sums go
    through three scan levels; samples equal the integer model exactly."""
    n = 25
    rng = np.random.default_rng(25)
    qs = new_state(rt, n, np.float32)
    ops = [('g', 'H', (), False, q, ()) for q in range(n)]
    ops += random_ops(rng, n, 20, max_controls=1)
    apply_ops(qs, ops)
    getter = rt.create_qubits_states_getter(np.float32)
    lanes = [(qs, [Lane(l, l) for l in range(n)])]
    probs = np.empty(1 << n, np.float32)
    getter.get_states(probs, 0, abs2, lanes, [], 1 << n, 0, 1)
    u = np.concatenate([rng.random(20000), EDGE_U])
    pool = getter.create_sampling_pool(list(range(n)), n, 0, lanes, [])
    got = np.asarray(pool.sample(len(u), u).intarray)
    pool.delete()
    qs.delete()
    assert np.array_equal(got, fixed_point_samples(probs, u))


@pytest.mark.parametrize('n, n_h, flips', [(14, 0, [3]), (20, 12, [15]), (25, 17, [20])],
                         ids=['basis14', 'h12of20', 'h17of25'])
def test_sampling_pool_guide_long_runs(rt, n, n_h, flips):
    """States whose items each span many guide buckets: a basis state (one
    item covers every bucket), H on 12 of 20 lanes (4096 items of 16
    buckets: the bounded list of long runs) and H on 17 of 25 lanes (2^17
    long runs: more than the list holds, so the pool searches without the
    table).  Samples equal the integer model exactly."""
    qs = new_state(rt, n, np.float32)
    ops = [('g', 'H', (), False, q, ()) for q in range(n_h)]
    ops += [('g', 'X', (), False, q, ()) for q in flips]
    apply_ops(qs, ops)
    getter = rt.create_qubits_states_getter(np.float32)
    lanes = [(qs, [Lane(l, l) for l in range(n)])]
    probs = np.empty(1 << n, np.float32)
    getter.get_states(probs, 0, abs2, lanes, [], 1 << n, 0, 1)
    rng = np.random.default_rng(n)
    u = np.concatenate([rng.random(20000), EDGE_U, (np.arange(64) + 0.5) / 64])
    pool = getter.create_sampling_pool(list(range(n)), n, 0, lanes, [])
    got = np.asarray(pool.sample(len(u), u).intarray)
    pool.delete()
    qs.delete()
    assert np.array_equal(got, fixed_point_samples(probs, u))
    if n_h == 0:  # uniforms in [0, 1) select the basis state; >= 1: n - 1; < 0, NaN: 0
        ok = (u >= 0.) & (u < 1.)
        assert np.all(got[ok] == sum(1 << q for q in flips))
        assert np.all(got[u >= 1.] == (1 << n) - 1) and np.all(got[~(u >= 0.)] == 0)


@pytest.mark.parametrize('k', [1, 3])
def test_sampling_pool_shifted_guide_entries(rt, k):
    """The guide layout of pools above 2^32 items (entries = item >> k,
    buckets of ~64 items), forced on a 20-qubit random state and on a basis
    state: samples equal the integer model exactly."""
    from qgate_gb300 import _native as nat
    n = 20
    rng = np.random.default_rng(30 + k)
    getter = rt.create_qubits_states_getter(np.float32)
    nat.call('qg_set_pool_guide_index_shift', k)
    try:
        for ops in (random_ops(rng, n, 40, max_controls=1), [('g', 'X', (), False, 7, ())]):
            qs = new_state(rt, n, np.float32)
            apply_ops(qs, ops)
            lanes = [(qs, [Lane(l, l) for l in range(n)])]
            probs = np.empty(1 << n, np.float32)
            getter.get_states(probs, 0, abs2, lanes, [], 1 << n, 0, 1)
            u = np.concatenate([rng.random(50000), EDGE_U])
            pool = getter.create_sampling_pool(list(range(n)), n, 0, lanes, [])
            got = np.asarray(pool.sample(len(u), u).intarray)
            pool.delete()
            qs.delete()
            assert np.array_equal(got, fixed_point_samples(probs, u))
    finally:
        nat.call('qg_set_pool_guide_index_shift', -1)


def test_sampling_pool_rejects_unnormalised_state(rt):
    """|sum - 1| > 0.05 raises, as CPUSamplingPool does
    (qgate/simulator/src/CPUSamplingPool.cpp:31-32)."""
    qs = new_state(rt, 4, np.float64)
    # decohere with a wrong probability leaves the state unnormalised
    qs.processor.decohere(0, 0.5, qs, 0)
    getter = rt.create_qubits_states_getter(np.float64)
    lt = _lane_trans([qs], [list(range(4))])
    with pytest.raises(RuntimeError, match='beyond 0.05'):
        getter.create_sampling_pool(list(range(4)), 4, 0, lt, [])


def test_direct_host_writes_match_staged(rt):
    """Getter outputs written by the kernels straight into the caller's
    pageable buffers (opt-in where the device supports it) equal the
    pinned-staging path bit for bit: probability vector and gathered states
    with lane permutation."""
    from qgate_gb300 import _native as nat
    info = nat.device_info()
    if not (info['pageable_memory_access'] and info['pageable_uses_host_page_tables']):
        pytest.skip('device does not access pageable host memory')
    rng = np.random.default_rng(5)
    n = 20
    ops = random_ops(rng, n, 40, max_controls=2)
    out = {}
    try:
        for direct in (1, 0):
            nat.call('qg_set_host_direct', direct)
            for dtype in (np.float32, np.float64):
                qs = new_state(rt, n, dtype)
                apply_ops(qs, ops)
                getter = rt.create_qubits_states_getter(dtype)
                probs = np.empty(1 << n, dtype)
                getter.get_states(probs, 0, abs2, [(qs, [Lane(l, (l * 7) % n) for l in range(n)])],
                                  [], 1 << n, 0, 1)
                cdt = np.complex64 if dtype == np.float32 else np.complex128
                amps = np.empty(1 << 12, cdt)
                getter.get_states(amps, 0, null, [(qs, [Lane(l, l) for l in range(n)])], [],
                                  1 << 12, 5, 3)
                out[(direct, dtype)] = (probs, amps)
                qs.delete()
    finally:
        nat.call('qg_set_host_direct', 0)
    for dtype in (np.float32, np.float64):
        for a, b in zip(out[(1, dtype)], out[(0, dtype)]):
            assert np.array_equal(a, b)


def test_pageable_copy_matches_staged(rt):
    """Large getter results (>= 64 MiB) go through one device buffer and one
    copy into the caller's pageable array where the device supports it (the
    default there); they equal the pinned-staging path bit for bit: a 24-qubit
    complex64 probability vector (64 MiB) and the state itself (128 MiB),
    into fresh and reused arrays."""
    from qgate_gb300 import _native as nat
    info = nat.device_info()
    if not (info['pageable_memory_access'] and info['pageable_uses_host_page_tables']):
        pytest.skip('device does not access pageable host memory')
    rng = np.random.default_rng(24)
    n = 24
    ops = random_ops(rng, n, 30, max_controls=1)
    qs = new_state(rt, n, np.float32)
    apply_ops(qs, ops)
    getter = rt.create_qubits_states_getter(np.float32)
    lanes = [(qs, [Lane(l, l) for l in range(n)])]
    out = {}
    try:
        for pc in (1, 0):
            nat.call('qg_set_pageable_copy', pc)
            probs = np.empty(1 << n, np.float32)
            getter.get_states(probs, 0, abs2, lanes, [], 1 << n, 0, 1)
            again = probs.copy()
            getter.get_states(again, 0, abs2, lanes, [], 1 << n, 0, 1)
            out[pc] = (probs, again, qs.get_raw())
    finally:
        nat.call('qg_set_pageable_copy', 1)
    for a, b in zip(out[1], out[0]):
        assert np.array_equal(a, b)
    assert np.array_equal(out[1][0], out[1][1])
    qs.delete()
