"""Speed of the oracle's C port against the reference's own C++ CPU runtime.

TEST INFRASTRUCTURE ONLY.  The benchmark's CPU baseline and reference arm
time the C port (oracle/cpu_statevec.c) because the reference's runtime
cannot run where the GPU is (its sources are not there).  This script runs
both here, where the reference builds (`make -C oracle ref`), on the same
gates and state, and prints their gate-pass rates side by side, so that the
port's figure can be read as the reference's.

    python oracle/port_speed.py [--qubits 26] [--threads N]

The gates are the first layer of the benchmark circuit (U3 on every qubit,
then CX on a seeded random matching), complex64; each gate counts the bytes
of its standalone read+write sweep.  The reference applies them through its
processor API (qgate/simulator/native_qubit_processor.py:50-59, into
CPUQubitProcessor.cpp:307-362) with its own thread pool
(qgate/simulator/src/Parallel.cpp:21-40, QGATE_NUM_WORKERS)."""
import argparse
import math
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def first_layer(n, seed=1):
    rng = np.random.default_rng(seed)
    ang = rng.uniform(0, 2 * math.pi, (n, 3))
    ops = [('U', tuple(float(x) for x in ang[q]), q, ()) for q in range(n)]
    perm = rng.permutation(n)
    ops += [('X', (), int(perm[2 * k + 1]), (int(perm[2 * k]),)) for k in range(n // 2)]
    return ops


def pass_bytes(n, ops, cs=8):
    return sum(2 * (1 << (n - len(c))) * cs for _, _, _, c in ops)


def time_port(n, ops, reps):
    from oracle import cpu_port, statevec as sv
    st = cpu_port.State(n, np.complex64)
    mats = [sv.gate_matrix(nm, a) for nm, a, _, _ in ops]
    for m, (_, _, t, c) in zip(mats, ops):  # warm-up (page faults)
        st.apply(m, t, c)
    t0 = time.perf_counter()
    for _ in range(reps):
        for m, (_, _, t, c) in zip(mats, ops):
            st.apply(m, t, c)
    return (time.perf_counter() - t0) / reps, cpu_port.num_threads()


def time_reference(n, ops, reps):
    from oracle.ref_import import import_reference
    qgate = import_reference()
    import qgate.model.gate_type as gtype
    import qgate.simulator.cpuruntime as cpuruntime
    qs = cpuruntime.create_qubit_states(np.float32)
    proc = qs.processor
    proc.initialize_qubit_states(qs, n)
    proc.reset_qubit_states(qs)
    gts = []
    for nm, a, t, c in ops:
        g = gtype.U(*a) if nm == 'U' else gtype.X()
        gts.append((g, t, list(c)))

    def run():
        for g, t, c in gts:
            if c:
                proc.apply_controlled_gate(g, False, qs, c, t)
            else:
                proc.apply_gate(g, False, qs, t)
        proc.synchronize()
    run()  # warm-up
    t0 = time.perf_counter()
    for _ in range(reps):
        run()
    return (time.perf_counter() - t0) / reps


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--qubits', type=int, default=26)
    ap.add_argument('--reps', type=int, default=3)
    ap.add_argument('--threads', type=int, default=os.cpu_count())
    args = ap.parse_args()
    os.environ.setdefault('QGATE_NUM_WORKERS', str(args.threads))
    os.environ.setdefault('OMP_NUM_THREADS', str(args.threads))
    n = args.qubits
    ops = first_layer(n)
    nbytes = pass_bytes(n, ops)
    t_port, thr = time_port(n, ops, args.reps)
    t_ref = time_reference(n, ops, args.reps)
    print('2^%d complex64, %d gates (%d U3 + %d CX), %d threads' %
          (n, len(ops), n, n // 2, thr))
    print('  reference CPU runtime: %.3f s per layer, %.1f GB/s gate-pass' %
          (t_ref, nbytes / t_ref / 1e9))
    print('  oracle C port        : %.3f s per layer, %.1f GB/s gate-pass' %
          (t_port, nbytes / t_port / 1e9))
    print('  port / reference     : %.2f' % (t_ref / t_port))


if __name__ == '__main__':
    main()
