"""GPU parity of the gate, reduction and measurement kernels against the oracle
(oracle/statevec.py, itself pinned to the reference).

Tolerances: complex128 1e-12 absolute on amplitudes / probabilities;
complex64 2e-6 absolute (FP32 amplitudes, FP64 accumulation)."""
import numpy as np
import pytest

from oracle import statevec as sv
from tests.gpu_helpers import (ATOL, CDT, apply_ops, fidelity_error, make_gate_type,
                               new_state, random_ops)

pytestmark = pytest.mark.gpu

DTYPES = [np.float64, np.float32]
IDS = ['c128', 'c64']


@pytest.fixture(autouse=True)
def default_fusion():
    from qgate_gb300 import _native as nat
    nat.set_fusion(0)
    yield
    nat.set_fusion(0)


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_single_gate_every_lane(rt, dtype):
    """Each lane of n=1..11 as target: covers the paired-float4, in-vector
    (lane 0) and complex128 pair kernels."""
    from qgate_gb300 import _native as nat
    nat.set_fusion(1)
    rng = np.random.default_rng(0)
    for n in range(1, 12):
        for lane in range(n):
            pre = random_ops(rng, n, 6, p_ctrl=0.)
            op = ('g', 'U', tuple(rng.uniform(0, 6, 3)), False, lane, ())
            qs = new_state(rt, n, dtype)
            apply_ops(qs, pre + [op])
            want = sv.run_ops(n, pre + [op], CDT[dtype])
            got = qs.get_raw()
            assert np.allclose(got, want, atol=ATOL[dtype]), (n, lane)


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_controlled_gates_all_patterns(rt, dtype):
    """Every (control, target) pair and 2-3 controls including lane 0 as a
    control (scalar kernel) and as target (in-vector kernel)."""
    from qgate_gb300 import _native as nat
    nat.set_fusion(1)
    rng = np.random.default_rng(1)
    n = 6
    pre = random_ops(rng, n, 12, p_ctrl=0.)
    cases = [(c, t) for c in range(n) for t in range(n) if c != t]
    cases = [((c,), t) for c, t in cases] + [((0, 3), 5), ((2, 4), 0), ((1, 5, 3), 2),
                                              ((0, 1, 2, 3, 4), 5)]
    for ctrls, t in cases:
        op = ('g', 'U', tuple(rng.uniform(0, 6, 3)), True, t, ctrls)
        qs = new_state(rt, n, dtype)
        apply_ops(qs, pre + [op])
        want = sv.run_ops(n, pre + [op], CDT[dtype])
        assert np.allclose(qs.get_raw(), want, atol=ATOL[dtype]), (ctrls, t)


@pytest.mark.parametrize('tile', [1, 2, 3, 5, 6, 8, 10, 12, 13])
@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_fused_stages_match_unfused(rt, dtype, tile):
    """Random circuits with 1-3 controls through the fusion planner at several
    tile widths (1 = off) on states smaller and larger than the tile."""
    from qgate_gb300 import _native as nat
    nat.set_fusion(tile)
    rng = np.random.default_rng(100 + tile)
    for n in (3, 7, 12, 15):
        ops = random_ops(rng, n, 60, max_controls=3)
        qs = new_state(rt, n, dtype)
        apply_ops(qs, ops)
        want = sv.run_ops(n, ops, CDT[dtype])
        got = qs.get_raw()
        tol = ATOL[dtype] * (4 if dtype == np.float32 else 1)
        assert np.allclose(got, want, atol=tol), (n, tile, np.max(np.abs(got - want)))


def _structured_circuits(rng, n):
    """Dense random gates with up to 3 controls; a QFT-like ladder of
    controlled phases (diagonal gates, many on thread lanes); CX-heavy layers
    of U3 + random matchings; merged single-lane runs (Ry then Rz)."""
    dense = random_ops(rng, n, 120, max_controls=3)
    qft = []
    for i in range(n):
        qft.append(('g', 'H', (), False, i, ()))
        for j in range(i + 1, n):
            qft.append(('g', 'U1', (np.pi / (1 << (j - i)),), False, i, (j,)))
    layers = []
    for _ in range(3):
        layers += [('g', 'U', tuple(rng.uniform(0, 6, 3)), False, q, ()) for q in range(n)]
        p = rng.permutation(n)
        layers += [('g', 'X', (), False, int(p[2 * k + 1]), (int(p[2 * k]),))
                   for k in range(n // 2)]
        layers += [('g', 'RY', (float(rng.uniform(-3, 3)),), False, q, ()) for q in range(n)]
        layers += [('g', 'RZ', (float(rng.uniform(-3, 3)),), False, q, ()) for q in range(n)]
    return [dense, qft, layers]


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_register_stage_shapes(rt, dtype):
    """The register-resident stage kernel at every valid (tile lanes,
    register lanes) shape, with and without a cost budget, on dense,
    diagonal-heavy and CX-heavy circuits (n = 16, so tiles < state)."""
    from qgate_gb300 import _native as nat
    prec = nat.PREC_FP64 if dtype == np.float64 else nat.PREC_FP32
    rng = np.random.default_rng(42)
    n = 16
    circuits = _structured_circuits(rng, n)
    wants = [sv.run_ops(n, ops, np.complex128) for ops in circuits]
    rls = (3, 4) if dtype == np.float64 else (3, 4, 5)
    tol = 1e-11 if dtype == np.float64 else 1e-5
    nat.set_tensor_blocks(False)  # this test covers the CUDA-core stage kernel
    try:
        for tile in (6, 8, 9, 10, 11, 12, 13):
            for rl in rls:
                for budget in (0, 40):
                    nat.set_fusion_params(prec, tile, rl, budget)
                    for ops, want in zip(circuits, wants):
                        qs = new_state(rt, n, dtype)
                        apply_ops(qs, ops)
                        got = qs.get_raw()
                        err = np.max(np.abs(got - want))
                        assert err < tol, (tile, rl, budget, err)
                        qs.delete()
    finally:
        nat.set_fusion(0)


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_pipelined_stage_kernel_22q(rt, dtype):
    """The persistent double-buffered stage kernel (used once a state has
    >= 304 tiles): 22 qubits, several tile shapes, against the oracle and
    against the one-CTA-per-tile kernel (bit-identical: same arithmetic)."""
    from qgate_gb300 import _native as nat
    prec = nat.PREC_FP64 if dtype == np.float64 else nat.PREC_FP32
    rng = np.random.default_rng(22)
    n = 22
    ops = random_ops(rng, n, 90, max_controls=2)
    want = sv.run_ops(n, ops, np.complex128)
    tol = 1e-11 if dtype == np.float64 else 1e-5
    shapes = [(11, 4), (12, 4), (13, 4)] + ([(12, 5), (13, 5)] if dtype == np.float32 else [])
    nat.set_tensor_blocks(False)  # this test covers the CUDA-core stage kernel
    try:
        for tile, rl in shapes:
            nat.set_fusion_params(prec, tile, rl, 0)
            got = {}
            for pipe in (1, 0):
                nat.call('qg_set_stage_pipelining', pipe)
                qs = new_state(rt, n, dtype)
                apply_ops(qs, ops)
                got[pipe] = qs.get_raw()
                qs.delete()
            assert np.max(np.abs(got[1] - want)) < tol, (tile, rl)
            assert np.array_equal(got[1], got[0]), (tile, rl)
    finally:
        nat.call('qg_set_stage_pipelining', 0)
        nat.set_fusion(0)


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_random_circuit_20q_fidelity(rt, dtype):
    """20 qubits, U3 layers + CX matchings (the 30-qubit benchmark circuit's
    structure at a size the oracle finishes in seconds)."""
    rng = np.random.default_rng(7)
    n, depth = 20, 4
    ops = []
    for _ in range(depth):
        ang = rng.uniform(0, 2 * np.pi, (n, 3))
        ops += [('g', 'U', tuple(ang[q]), False, q, ()) for q in range(n)]
        perm = rng.permutation(n)
        ops += [('g', 'X', (), False, int(perm[2 * k + 1]), (int(perm[2 * k]),))
                for k in range(n // 2)]
    qs = new_state(rt, n, dtype)
    apply_ops(qs, ops)
    want = sv.run_ops(n, ops, np.complex128)
    got = qs.get_raw()
    ferr = fidelity_error(want, got)
    perr = np.max(np.abs(np.abs(got.astype(np.complex128)) ** 2 - np.abs(want) ** 2))
    if dtype == np.float64:
        assert ferr < 1e-12 and perr < 1e-14
    else:
        assert ferr < 1e-5 and perr < 1e-7, (ferr, perr)


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_calc_probability_and_norm(rt, dtype):
    rng = np.random.default_rng(3)
    for n in (1, 2, 5, 13):
        ops = random_ops(rng, n, 30)
        qs = new_state(rt, n, dtype)
        apply_ops(qs, ops)
        psi = sv.run_ops(n, ops, np.complex128)
        tol = 1e-12 if dtype == np.float64 else 2e-6
        for lane in range(n):
            p = qs.processor.calc_probability(qs, lane)
            assert abs(p - sv.calc_probability(psi, lane)) < tol
        assert abs(qs.processor.calc_norm(qs) - 1.) < tol


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_pauli_expectation(rt, dtype):
    """<P> on random states; also the reference relation Pr(+1) = (1+<P>)/2
    for Z strings (qgate/model/pauli_gates_diagonalizer.py)."""
    rng = np.random.default_rng(4)
    n = 9
    ops = random_ops(rng, n, 80)
    qs = new_state(rt, n, dtype)
    apply_ops(qs, ops)
    psi = sv.run_ops(n, ops, np.complex128)
    tol = 1e-12 if dtype == np.float64 else 3e-6
    for _ in range(40):
        x = int(rng.integers(0, 1 << n))
        z = int(rng.integers(0, 1 << n))
        got = qs.processor.calc_pauli_expectation(qs, x, z)
        assert abs(got - sv.pauli_expectation(psi, x, z)) < tol, (x, z)
    for lane in range(n):
        pz = qs.processor.calc_pauli_expectation(qs, 0, 1 << lane)
        assert abs((1 + pz) / 2 - sv.calc_probability(psi, lane)) < tol


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_apply_matrix_multi_target(rt, dtype):
    """Dense k-target gates vs the oracle; SWAP as a 2-target matrix equals the
    reference's 3-CX expansion (qgate/model/expand.py:14-16)."""
    rng = np.random.default_rng(5)
    n = 8
    for k in (1, 2, 3, 4, 5):
        m = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
        u, _ = np.linalg.qr(m)
        targets = [int(t) for t in rng.permutation(n)[:k]]
        rest = [q for q in range(n) if q not in targets]
        ctrls = [rest[0]] if k <= 3 else []
        pre = random_ops(rng, n, 20)
        qs = new_state(rt, n, dtype)
        apply_ops(qs, pre)
        qs.processor.apply_matrix(u, qs, targets, ctrls)
        psi = sv.run_ops(n, pre, np.complex128)
        sv.apply_matrix(psi, u, targets, ctrls)
        assert np.allclose(qs.get_raw(), psi, atol=ATOL[dtype] * 4), k
    swap = np.eye(4)[[0, 2, 1, 3]]
    pre = random_ops(rng, n, 20)
    qs = new_state(rt, n, dtype)
    apply_ops(qs, pre)
    qs.processor.apply_matrix(swap, qs, [2, 6])
    three_cx = [('g', 'X', (), False, 6, (2,)), ('g', 'X', (), False, 2, (6,)),
                ('g', 'X', (), False, 6, (2,))]
    want = sv.run_ops(n, pre + three_cx, np.complex128)
    assert np.allclose(qs.get_raw(), want, atol=ATOL[dtype])


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_measure_decohere_reset(rt, dtype):
    rng = np.random.default_rng(6)
    n = 7
    for lane in range(n):
        for value in (0, 1):
            ops = random_ops(rng, n, 25)
            qs = new_state(rt, n, dtype)
            apply_ops(qs, ops)
            psi = sv.run_ops(n, ops, np.complex128)
            p = sv.calc_probability(psi, lane)
            qs.processor.decohere(value, p, qs, lane)
            sv.decohere(psi, value, p, lane)
            assert np.allclose(qs.get_raw(), psi, atol=ATOL[dtype] * 4)
            if value == 1:
                qs.processor.apply_reset(qs, lane)
                sv.apply_reset(psi, lane)
                assert np.allclose(qs.get_raw(), psi, atol=ATOL[dtype] * 4)


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_decohere_and_separate(rt, dtype):
    rng = np.random.default_rng(8)
    n = 6
    for lane in range(n):
        for value in (0, 1):
            ops = random_ops(rng, n, 25)
            qs = new_state(rt, n, dtype)
            apply_ops(qs, ops)
            psi = sv.run_ops(n, ops, np.complex128)
            p = sv.calc_probability(psi, lane)
            qs0 = rt.create_qubit_states(dtype)
            qs1 = rt.create_qubit_states(dtype)
            qs.processor.initialize_qubit_states(qs0, n - 1)
            qs.processor.initialize_qubit_states(qs1, 1)
            qs.processor.decohere_and_separate(value, p, qs0, qs1, qs, lane)
            w0, w1 = sv.decohere_and_separate(psi, value, p, lane)
            assert np.allclose(qs0.get_raw(), w0, atol=ATOL[dtype] * 4)
            assert np.allclose(qs1.get_raw(), w1, atol=0)


@pytest.mark.parametrize('dtype', DTYPES, ids=IDS)
def test_join_kron(rt, dtype):
    rng = np.random.default_rng(9)
    sizes = [3, 1, 4, 2]
    parts, objs = [], []
    for k in sizes:
        ops = random_ops(rng, k, 10)
        qs = new_state(rt, k, dtype)
        apply_ops(qs, ops)
        objs.append(qs)
        parts.append(sv.run_ops(k, ops, np.complex128))
    for n_new in (0, 2):
        joined = rt.create_qubit_states(dtype)
        total = sum(sizes) + n_new
        joined.processor.initialize_qubit_states(joined, total)
        joined.processor.join(joined, objs, n_new)
        want = sv.join(parts, n_new)
        assert np.allclose(joined.get_raw(), want, atol=ATOL[dtype] * 4)


def test_errors_are_raised_not_crashed(rt):
    qs = new_state(rt, 3, np.float64)
    with pytest.raises(ValueError):
        qs.processor.apply_gate(make_gate_type('H', ()), False, qs, 3)
    with pytest.raises(RuntimeError):
        qs.processor.apply_controlled_gate(make_gate_type('X', ()), False, qs, [1], 1)
    with pytest.raises(ValueError):
        qs.processor.calc_probability(qs, -1)
    with pytest.raises(RuntimeError, match='Unknown gate type'):
        qs.processor.apply_gate(make_gate_type('NOPE', ()), False, qs, 0)
    # the state is still usable after the errors
    qs.processor.apply_gate(make_gate_type('X', ()), False, qs, 2)
    assert abs(qs.processor.calc_probability(qs, 2)) < 1e-15


def test_arena_reuses_freed_states(rt):
    from qgate_gb300 import _native as nat
    before = nat.arena_stats()
    for _ in range(20):
        qs = new_state(rt, 16, np.float32)
        qs.delete()
    after = nat.arena_stats()
    assert after['in_use'] == before['in_use']
