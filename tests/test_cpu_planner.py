"""CPU checks of the tensor-stage host planner (tests/cpp/planner_check.cpp
built against qgate_gb300/csrc/tcplan.cpp with the host compiler): FP16
rounding of the block operands against numpy, the split operands' accuracy,
the stage planner's partition and commutation safety, the fast gate count
against stage_take, fused-block limits, and that every operand slot table is
a bijection onto the 4096 slots of a tile (what the tensor-core kernel's
shared-memory staging relies on); and (tests/cpp/plan_count.cpp) the pass and
block counts of the bench circuits' tensor-stage plans."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, 'qgate_gb300', 'csrc')


def _cuda_include():
    for base in (os.environ.get('CUDA_HOME'), '/usr/local/cuda'):
        if base and os.path.exists(os.path.join(base, 'include', 'cuda_runtime.h')):
            return os.path.join(base, 'include')
    return None


@pytest.fixture(scope='module')
def planner_run(tmp_path_factory):
    cxx = shutil.which('g++')
    inc = _cuda_include()
    if not cxx or not inc:
        pytest.skip('needs g++ and the CUDA headers')
    d = tmp_path_factory.mktemp('planner')
    exe = str(d / 'planner_check')
    subprocess.run([cxx, '-O1', '-std=c++17', '-fopenmp', '-I', CSRC, '-I',
                    os.path.join(ROOT, 'include'), '-I', inc,
                    os.path.join(ROOT, 'tests', 'cpp', 'planner_check.cpp'), '-o', exe],
                   check=True, capture_output=True)
    pairs = str(d / 'f16.bin')
    out = subprocess.run([exe, pairs], check=True, capture_output=True, text=True).stdout
    vals = dict(line.split() for line in out.strip().splitlines())
    return vals, pairs


def test_fp16_rounding_matches_numpy(planner_run):
    _, pairs = planner_run
    rec = np.fromfile(pairs, dtype=np.dtype([('x', '<f4'), ('h', '<u2')]))
    want = rec['x'].astype(np.float16).view(np.uint16)
    assert np.array_equal(rec['h'], want)


def test_split_operands_accuracy(planner_run):
    vals, _ = planner_run
    # FP16 hi + FP16 lo of entries <= 1: error below 2^-22 (relative) + lo's own rounding
    assert float(vals['operand_split_max_abs_err']) < 2. ** -21


def test_stage_planner_invariants(planner_run):
    """Stage lane sets, gate partitions and fused blocks on random gate lists,
    half of them with cross gates allowed (diagonal gates with at most one
    lane in the tile, taken as per-tile phases): taken gates fit the tile or
    are cross gates, nothing moves past a deferred gate it shares a lane with,
    and blocks reorder gates only where they commute."""
    vals, _ = planner_run
    for k in ('bad_partition', 'bad_commute', 'bad_count', 'bad_lanes', 'bad_blocks'):
        assert int(vals[k]) == 0, k
    assert int(vals['cross_taken']) > 0


def test_operand_slot_tables_are_bijections(planner_run):
    vals, _ = planner_run
    assert int(vals['bad_slots']) == 0
    assert int(vals['bad_tables']) == 0
    assert int(vals['launches_checked']) >= 5


def test_emulated_stage_matches_the_gates(planner_run):
    """The tensor-stage kernel's data flow emulated in FP64 from launch plans
    (load layout, slot tables, Bh + Bl operands, phase tables or cross
    records, natural tile or the direct row stores)
    equals the plans' gates applied to the tile, for 12- and 13-lane tiles
    with dense and phase ops; what remains is the operands' FP16 split (~2^-22
    per op) and the compensation scale (~1e-7 per dense op)."""
    vals, _ = planner_run
    assert float(vals['emulated_stage_max_rel_err']) < 5e-6
    assert int(vals['phase_ops']) > 0 and int(vals['dense_ops']) > 0
    # launches that store rows straight to the state (their last dense block
    # leaves lanes 0 and 1 to the rows) and ones through the natural tile
    direct = int(vals['direct_out_launches'])
    assert 0 < direct < int(vals['launches_checked'])
    # cross ops (per-tile phases from gates with lanes outside the tile),
    # emulated on a tile with random bits outside it
    assert int(vals['cross_ops']) > 0


def _write_circuit(path, label, n, ops):
    from oracle import statevec as sv
    rows = []
    for name, args, target, ctrls in ops:
        m = np.asarray(sv.gate_matrix(name, args), np.complex128).reshape(-1)
        vals = ' '.join('%r %r' % (float(z.real), float(z.imag)) for z in m)
        rows.append('%d %d %s %s' % (target, len(ctrls), ' '.join(map(str, ctrls)), vals))
    with open(path, 'w') as f:
        f.write('%s %d %d\n%s\n' % (label, n, len(rows), '\n'.join(rows)))


def test_bench_circuit_plans(tmp_path):
    """Pass and block counts of the complex64 tensor-stage plans of the bench's
    circuits (tests/cpp/plan_count.cpp: the gate queue's merge of runs, then
    its lookahead stage planner and the fused-block grouping per stage, on
    12-lane tiles): the 30-qubit, depth-20 random U3+CX circuit in 32 passes of
    97 dense blocks; the 33-qubit, depth-30 one (seeds 40) in 54 passes; the
    34-qubit QFT in 4 passes and the 20-qubit one in 2, both as the queue sees
    them once the X gates of their input preparation have folded into the reset
    basis state (their controlled phases then run as per-tile phase and cross
    ops)."""
    import bench
    cxx = shutil.which('g++')
    inc = _cuda_include()
    if not cxx or not inc:
        pytest.skip('needs g++ and the CUDA headers')
    exe = str(tmp_path / 'plan_count')
    subprocess.run([cxx, '-O2', '-std=c++17', '-fopenmp', '-I', CSRC, '-I',
                    os.path.join(ROOT, 'include'), '-I', inc,
                    os.path.join(ROOT, 'tests', 'cpp', 'plan_count.cpp'), '-o', exe],
                   check=True, capture_output=True)
    cases = [('random30', 30, bench.circuit(30, 20)),
             ('random33', 33, bench.circuit(33, 30, seed_angles=40, seed_perm=40)),
             ('qft34', 34, [o for o in bench.qft_ops(34, 41) if o[0] != 'X']),
             ('qft20', 20, [o for o in bench.qft_ops(20, 0) if o[0] != 'X'])]
    files = []
    for label, n, ops in cases:
        files.append(str(tmp_path / (label + '.txt')))
        _write_circuit(files[-1], label, n, ops)
    out = subprocess.run([exe] + files, check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.strip().splitlines():
        label, *nums = line.split()
        got[label] = dict(zip(('gates', 'passes', 'single', 'dense', 'phase', 'cross'),
                              map(int, nums)))
    assert got['random30'] == dict(gates=900, passes=32, single=0, dense=97, phase=0, cross=0)
    assert got['random33']['passes'] == 54 and got['random33']['single'] == 0
    assert got['qft34'] == dict(gates=595, passes=4, single=0, dense=9, phase=5, cross=3)
    assert got['qft20']['passes'] == 2 and got['qft20']['cross'] >= 1
