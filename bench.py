#!/usr/bin/env python
"""Benchmark of the GB300 state-vector engine on the 30-qubit random circuit.

Workload (the headline configuration): 30 qubits, depth 20; each layer applies
U3(theta, phi, lambda) to every qubit with angles uniform in [0, 2pi)
(numpy default_rng(10), shape (20, 30, 3)), then CX on a random perfect
matching of the qubits (default_rng(11).permutation(30) per layer: pairs
(p[2k], p[2k+1]), control first).  complex64 by default (--dtype c128 for
complex128).  Inputs are synthetic; the state (8 GiB in complex64) is far
larger than the 129 MB L2, so no L2 flush is needed between steps.

A step = reset the resident state to |0...0> and run the 900-gate circuit
through the runtime plugin API (gates are queued, fused into shared-memory
stages and launched at synchronize).  `value` = gate-pass bytes per second of
device time, where each gate counts the bytes the reference moves for it as a
standalone pass (one read + one write of every amplitude it touches, the
unfused sweep of qgate/simulator/src/DeviceProcPrimitives.cu:198-249); the
same definition as the `--impl reference` arm, which runs those passes one by
one.  Fused stages apply many gates per HBM pass, so `value` can exceed the
HBM bandwidth; the bytes the engine actually moves, and the per-launch
roofline of the dominant kernel, are reported beside it (`config`,
`roofline`), as is the HBM efficiency of a single unfused gate pass.
`e2e` = the same gate-pass bytes per second of a step that also brings the
circuit's outputs to the host through the plugin API: the full probability
vector and 1e7 samples drawn from pre-drawn uniforms.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

`--impl reference` times the reference's CPU algorithm (the oracle's C port
of the reference CPU runtime, all host threads) on the same workload and
metric, on a bounded sample of the circuit's gates per step.
"""
import argparse
import json
import math
import os
import statistics
import platform
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = '30q gate-pass GB/s'
L2_BYTES = 129 << 20  # GB300 L2 (a state larger than this streams from HBM every step)


def circuit(n, depth, seed_angles=10, seed_perm=11):
    """[(name, args, target, controls)] of the random U3 + CX circuit."""
    ang = np.random.default_rng(seed_angles).uniform(0, 2 * math.pi, (depth, n, 3))
    prng = np.random.default_rng(seed_perm)
    ops = []
    for layer in range(depth):
        ops += [('U', tuple(float(a) for a in ang[layer, q]), q, ()) for q in range(n)]
        p = prng.permutation(n)
        ops += [('X', (), int(p[2 * k + 1]), (int(p[2 * k]),)) for k in range(n // 2)]
    return ops


def gate_pass_bytes(n, ops, cs):
    """Unfused algorithmic bytes: each gate reads and writes the amplitudes it
    touches (2^(n - #controls))."""
    return sum(2 * (1 << (n - len(c))) * cs for _, _, _, c in ops)


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.FIELDS,
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for line in self.lines:
            parts = [x.strip() for x in line.split(',')]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == 'active':
                    reasons.add(nm)
        return {'sm_mhz': statistics.median(sm) if sm else None,
                'sm_max_mhz': max(smax) if smax else None,
                'reasons': sorted(reasons), 'samples': len(sm)}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            return float(json.load(f)['hbm_gbs']), 'measured'
    except Exception:
        return 6800.0, 'fallback'


def stage_traffic_per_launch(n, cs, kernel_class='stage'):
    """DRAM bytes per fused-stage launch: bytes per amplitude from the ncu
    capture recorded in profiles/stage_traffic.txt (a smaller state, same
    kernel; traffic grows in proportion to the amplitudes), scaled to 2^n."""
    key = ('c64' if cs == 8 else 'c128') + ('_tensor' if kernel_class == 'tstage' else '')
    try:
        with open(os.path.join(ROOT, 'profiles', 'stage_traffic.txt')) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 3 and parts[0] == key and parts[1] == 'dram_bytes_per_amp':
                    return float(parts[2]) * (1 << n)
    except OSError:
        pass
    return None


# ------------------------------------------------------------------ CPU legs

def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo), for the CPU
    baseline's record."""
    try:
        out = subprocess.run(['lscpu'], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith('Model name:'):
                return line.split(':', 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open('/proc/cpuinfo') as f:
            for line in f:
                if line.startswith('model name'):
                    return line.split(':', 1)[1].strip()
    except OSError:
        pass
    return platform.machine()


def state_accuracy(rt, qs, gts, n, torch):
    """Fidelity error |1 - |<psi128|psi64>||, max |p64 - p128| and the
    complex64 norm of the benchmark circuit's final state (`qs`, complex64)
    against the same circuit run in complex128 by the engine (FP64 state,
    double-float register arithmetic), whose time is reported too.  Both states are copied to the host; the overlap is summed
    in FP64 in slices."""
    qd = rt.create_qubit_states(np.float64)
    pd = qd.processor
    pd.initialize_qubit_states(qd, n)
    pd.reset_qubit_states(qd)
    pd.synchronize()
    nat = sys.modules['qgate_gb300._native']
    nat.gate_stats(reset=True)
    t0 = time.perf_counter()
    for gt, t, c in gts:
        if c:
            pd.apply_controlled_gate(gt, False, qd, c, t)
        else:
            pd.apply_gate(gt, False, qd, t)
    pd.synchronize()
    c128_ms = (time.perf_counter() - t0) * 1e3
    st = nat.gate_stats(reset=True)
    ref = qd.get_raw()
    qd.delete()
    got = qs.get_raw()
    norm32 = qs.processor.calc_norm(qs)
    ov = 0j
    perr = 0.
    step = 1 << 24
    for i in range(0, 1 << n, step):
        a = torch.from_numpy(ref[i:i + step])
        b = torch.from_numpy(got[i:i + step]).to(torch.complex128)
        ov += torch.vdot(a, b).item()
        perr = max(perr, (a.abs() ** 2 - b.abs() ** 2).abs().max().item())
    return {'reference': 'the same circuit in complex128 (engine: FP64 state, double-float '
                         'register arithmetic)',
            'fidelity_err': abs(1. - abs(ov)), 'max_prob_err': perr, 'norm_c64': norm32,
            'c128_circuit_ms': c128_ms, 'c128_passes': st['passes'],
            'c128_hbm_gbs_actual': st['bytes'] / (c128_ms / 1e3) / 1e9,
            'c128_note': 'complex128 stages compute in double-float on the FP32 pipes '
                         '(GB300 runs ~2 FP64 operations per clock per SM); they stay '
                         'arithmetic-bound, not HBM-bound'}


def cpu_port_gate_rate(n, ops, cs, budget_s):
    """Times the oracle's C port of the reference CPU runtime on the first
    gates of the circuit until `budget_s` seconds are spent.  Returns
    (GB/s, gates timed, seconds, threads)."""
    from oracle import cpu_port, statevec as sv
    st = cpu_port.State(n, np.complex64 if cs == 8 else np.complex128)
    mats = {}
    done, nbytes = 0, 0
    t0 = time.perf_counter()
    for name, args, target, ctrls in ops:
        key = (name, args)
        if key not in mats:
            mats[key] = sv.gate_matrix(name, args)
        st.apply(mats[key], target, ctrls)
        done += 1
        nbytes += 2 * (1 << (n - len(ctrls))) * cs
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return nbytes / dt / 1e9, done, dt, cpu_port.num_threads(), st


def cpu_port_observations(st, samples):
    """Times the oracle's C port of the reference CPU runtime's observations
    on a host state, the classes `observation_kernels` times on the GPU: Pr
    of the highest lane (qgate/simulator/src/CPUQubitProcessor.cpp:75-125),
    the full probability vector (FP64 here; the reference's is in the
    state's precision), the sampling pool's normalised prefix sums
    (CPUSamplingPool.cpp:8-63, in place) and `samples` draws from
    default_rng(12) (CPUSamplingPool.cpp:71-81)."""
    from oracle import cpu_port
    n, amp = st.n, st.psi.itemsize
    N = 1 << n
    t0 = time.perf_counter()
    st.calc_probability(n - 1)
    t_prob = time.perf_counter() - t0
    t0 = time.perf_counter()
    probs = st.probabilities()
    t_vec = time.perf_counter() - t0
    t0 = time.perf_counter()
    cdf, _ = cpu_port.prefix_cdf(probs, copy=False)
    t_pool = time.perf_counter() - t0
    u = np.random.default_rng(12).random(samples)
    t0 = time.perf_counter()
    cpu_port.sample_cdf(cdf, u)
    t_samp = time.perf_counter() - t0
    del probs, cdf
    return {'prob': {'ms': t_prob * 1e3, 'gbs': N // 2 * amp / t_prob / 1e9},
            'probability_vector': {'ms': t_vec * 1e3, 'gbs': (N * amp + N * 8) / t_vec / 1e9},
            'pool_prefix_sums': {'ms': t_pool * 1e3, 'gbs': 2 * N * 8 / t_pool / 1e9},
            'sample': {'samples': samples, 'ms': t_samp * 1e3, 'samples_per_s': samples / t_samp},
            'threads': cpu_port.num_threads()}


def run_reference(args):
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return
    n, cs = args.qubits, 16 if args.dtype == 'c128' else 8
    ops = circuit(n, args.depth)
    from oracle import cpu_port, statevec as sv
    st = cpu_port.State(n, np.complex64 if cs == 8 else np.complex128)
    sample = ops[:args.ref_gates]
    mats = [sv.gate_matrix(nm, a) for nm, a, _, _ in sample]
    step_bytes = gate_pass_bytes(n, sample, cs)
    for _ in range(args.warmup):
        for m, (_, _, t, c) in zip(mats, sample):
            st.apply(m, t, c)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for m, (_, _, t, c) in zip(mats, sample):
            st.apply(m, t, c)
    dt = time.perf_counter() - t0
    value = step_bytes * args.steps / dt / 1e9
    observations = cpu_port_observations(st, args.samples)  # after the timed steps
    n_cx = sum(1 for _, _, _, c in sample if c)
    sample_desc = ('first %d gates of the circuit (%d U3 + %d CX) per step on a 2^%d %s state '
                   'in host memory; the port runs at about the reference CPU runtime\'s own '
                   'rate (oracle/port_speed.py on two x86 build hosts: port/reference '
                   '0.92-0.99x with 8 threads, 0.96-1.33x on one thread)'
                   % (len(sample), len(sample) - n_cx, n_cx, n, args.dtype))
    line = {
        'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': 'GB/s',
        'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': dt / args.steps * 1e3, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': args.dtype, 'data': 'synthetic',
        'config': config_block(args),
        'cpu_baseline': {'value': value, 'unit': 'GB/s', 'cores': cpu_port.num_threads(),
                         'cpu_model': cpu_model(),
                         'kind': 'port', 'sample': sample_desc,
                         'observations': observations},
        'e2e': {'value': value, 'unit': 'GB/s', 'h2d_bytes_per_step': 0,
                'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line), flush=True)


def config_block(args):
    """The workload and the metric's definition: the same object in both
    arms' lines (measured figures go elsewhere)."""
    return {'workload': 'random U3+CX circuit, %d qubits, depth %d, %s (layers: U3 on every '
                        'qubit, CX on a seeded random matching)' % (args.qubits, args.depth,
                                                                     args.dtype),
            'qubits': args.qubits, 'depth': args.depth,
            'gates': args.qubits * args.depth + (args.qubits // 2) * args.depth,
            'l2': ('state larger than L2 (no flush needed)'
                   if (1 << args.qubits) * (16 if args.dtype == 'c128' else 8) > L2_BYTES
                   else 'state fits in L2: steps run warm'),
            'parallelism': 'replicas',
            'value_definition': 'unfused gate-pass bytes (each gate as its own read+write '
                                'sweep of the amplitudes it touches) per second'}


# ------------------------------------------------------------------ GPU leg

def run_gb300(args):
    import torch
    from qgate_gb300 import replicas
    world, rank, local = replicas.init()
    torch.cuda.set_device(local)

    from qgate_gb300 import _native as nat
    from qgate_gb300 import gb300runtime as rt
    from qgate_gb300.circuit import gate_type, Lane, abs2

    rt.set_preference(device_ids=[local])
    n, cs = args.qubits, 16 if args.dtype == 'c128' else 8
    dtype = np.float64 if args.dtype == 'c128' else np.float32
    ops = circuit(n, args.depth)
    gts = [(gate_type(nm, *a), t, list(c)) for nm, a, t, c in ops]
    unfused_bytes = gate_pass_bytes(n, ops, cs)
    if args.tile == 0:
        from qgate_gb300 import autotune
        tuned = autotune.tune(n, dtype, ops, use_cache=not args.retune)
    else:
        nat.set_fusion(args.tile)
        tuned = {'tile_lanes': args.tile}
    if args.no_tensor:
        nat.set_tensor_blocks(False)
        tuned = dict(tuned, tensor=0)

    qs = rt.create_qubit_states(dtype)
    proc = qs.processor
    proc.initialize_qubit_states(qs, n)

    def step():
        proc.reset_qubit_states(qs)
        for gt, t, c in gts:
            if c:
                proc.apply_controlled_gate(gt, False, qs, c, t)
            else:
                proc.apply_gate(gt, False, qs, t)
        proc.synchronize()

    # Trace replay off for the timed circuit: every stage is its own timed
    # launch (with tensor stages the 900-gate circuit streams anyway, which
    # trace replay leaves alone; with --no-tensor it would replay one graph)
    nat.set_trace_replay(False)
    for _ in range(args.warmup):
        step()
    stream = torch.cuda.ExternalStream(nat.stream_handle())
    nat.gate_stats(reset=True)
    nat.timing_all(reset=True)
    sampler = ClockSampler(local)
    sampler.start()
    replicas.barrier()
    torch.cuda.synchronize()
    nat.timing_enable(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    nat.timing_enable(False)
    nat.set_trace_replay(True)
    clocks = sampler.stop()
    dev_ms = e0.elapsed_time(e1)
    stats = nat.gate_stats(reset=True)
    timing = nat.timing_all(reset=True)
    init_bytes = (1 << n) * cs * args.steps
    moved = stats['bytes'] + init_bytes
    value, t_max_s = replicas.aggregate_throughput(unfused_bytes * args.steps, dev_ms / 1e3)
    value /= 1e9
    t_max = t_max_s * 1e3
    hbm_actual = moved * world / (t_max / 1e3) / 1e9
    launches = sum(v[0] for v in timing.values())

    # roofline of the dominant kernel class
    dom = max(timing.items(), key=lambda kv: kv[1][1])
    dom_name, (dom_launches, dom_ms) = dom
    peak, peak_kind = measured_peak_hbm()
    if dom_name in ('stage', 'tstage'):
        alg = 2 * (1 << n) * cs
        traffic = stage_traffic_per_launch(n, cs, dom_name)
    else:
        alg = stats['bytes'] / max(1, stats['passes'])
        traffic = None
    achieved = alg / (dom_ms / dom_launches / 1e3) / 1e9 if dom_launches else 0.
    roofline = {'kernel': {'stage': 'k_rstage (fused register-resident stage)',
                           'tstage': 'k_tstage (fused 5-lane blocks on tcgen05 tensor cores)',
                           'gate': 'k_pairs (single gate)'}.get(dom_name, dom_name),
                'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
                'frac': achieved / peak, 'peak_source': peak_kind,
                'traffic': traffic, 'algorithmic_bytes_per_launch': alg,
                'launches': dom_launches, 'avg_launch_ms': dom_ms / max(1, dom_launches)}

    # accuracy of the timed state (the last step's) against the same circuit
    # in complex128
    accuracy = None
    if rank == 0 and dtype == np.float32 and not args.no_fidelity:
        accuracy = state_accuracy(rt, qs, gts, n, torch)

    # HBM efficiency of single unfused gate passes (the reference's per-gate sweep)
    single = single_gate_passes(nat, proc, qs, gts, n, cs, torch)

    # end to end through the plugin API with host buffers
    e2e = None
    if not args.no_e2e and rank == 0:
        e2e = run_e2e(args, rt, nat, qs, step, ops, n, cs, dtype, Lane, abs2)

    kernels = None
    if rank == 0 and not args.no_e2e:
        kernels = observation_kernels(args, rt, nat, proc, qs, n, cs, dtype, Lane, abs2)

    compiled = None
    if rank == 0 and not args.no_compiled:
        compiled = run_compiled(args, rt, nat)

    batch = None
    if rank == 0 and not args.no_batch:
        batch = run_batch(args, nat)


    adjoint = None
    if rank == 0 and not args.no_adjoint:
        qs.delete()
        adjoint = run_adjoint(args)

    c4 = None
    if rank == 0 and not args.no_c4:
        qs.delete()
        nat.call('qg_devices_clear')
        c4 = run_c4(args, rt, nat)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        gbs, done, dt, thr, st = cpu_port_gate_rate(n, ops, cs, args.cpu_seconds)
        cpu = {'value': gbs, 'unit': 'GB/s', 'cores': thr, 'kind': 'port', 'cpu_model': cpu_model(),
               'sample': 'first %d gates of the circuit on a 2^%d %s state in host memory, '
                         '%.1f s' % (done, n, args.dtype, dt),
               'observations': cpu_port_observations(st, args.samples)}
        del st

    if rank == 0:
        per_step_passes = stats['passes'] / args.steps
        line = {
            'metric': METRIC, 'value': value, 'unit': 'GB/s', 'n_gpus': world,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': t_max / args.steps,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': args.dtype, 'data': 'synthetic',
            'config': config_block(args),
            'step': {
                'fusion': {k: tuned.get(k) for k in ('tile_lanes', 'reg_lanes', 'cost_budget',
                                                    'tensor', 'prefetch')},
                'hbm_gbs_actual': hbm_actual,
                'single_gate_pass': single,
                'passes_per_step': per_step_passes,
                'gates_per_step': stats['gates'] / args.steps,
                'gate_pass_bytes_per_step': stats['bytes'] / args.steps,
                'unfused_gate_pass_bytes_per_step': unfused_bytes,
                'circuit_ms': t_max / args.steps,
                'gates_per_s': stats['gates'] / args.steps / (t_max / args.steps / 1e3)},
            'roofline': roofline,
            'observation_kernels': kernels,
            'compiled': compiled,
            'accuracy': accuracy,
            'adjoint': adjoint,
            'batch': batch,
            'large_states': c4,
            'cpu_baseline': cpu,
            'e2e': e2e,
            'gpu_launches': launches,
            'kernel_ms': {k: v[1] for k, v in timing.items() if v[0]},
            'clocks': clocks,
        }
        print(json.dumps(line), flush=True)
    replicas.finish()


def single_gate_passes(nat, proc, qs, gts, n, cs, torch, count=8):
    """Times `count` U3 gates of the circuit each as its own unfused pass
    (fusion off) on the resident state: the per-pass HBM efficiency of the
    single-gate kernel."""
    g1 = [g for g in gts if not g[2]][:count]
    stream = torch.cuda.ExternalStream(nat.stream_handle())
    saved = None
    try:
        nat.set_fusion_params(nat.PREC_FP32 if cs == 8 else nat.PREC_FP64, 1, 4, 0)
        saved = True
        for gt, t, c in g1:
            proc.apply_gate(gt, False, qs, t)
        proc.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for gt, t, c in g1:
            proc.apply_gate(gt, False, qs, t)
        proc.synchronize()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / len(g1)
    finally:
        if saved:
            from qgate_gb300 import autotune
            cached = autotune._load().get(autotune._key(n, np.float32 if cs == 8 else np.float64))
            if cached:
                autotune.apply(cached)
            else:
                nat.set_fusion(0)
    gbs = 2 * (1 << n) * cs / (ms / 1e3) / 1e9
    peak, kind = measured_peak_hbm()
    return {'kernel': 'k_pairs (one 2x2 gate per pass)', 'ms_per_pass': ms, 'gbs': gbs,
            'frac_of_peak': gbs / peak, 'peak_source': kind}


def run_adjoint(args):
    """Adjoint gradients of the 24-qubit hardware-efficient ansatz (12 layers
    of Ry, Rz on every qubit + CX ring, 576 parameters uniform(-pi, pi) from
    default_rng(30), batch of 64 vectors) for the transverse-field Ising chain
    H = -sum Z_i Z_{i+1} - 0.7 sum X_i, complex64 (checkpoints every 3 layers)
    and complex128; gradient vectors per second and the complex64 error
    against the complex128 gradients."""
    from qgate_gb300.adjoint import expectation_and_gradient, hardware_efficient_ansatz, PauliSum
    n, layers, B = args.adj_qubits, 12, args.adj_batch
    c = hardware_efficient_ansatz(n, layers)
    H = PauliSum.ising_chain(n)
    params = np.random.default_rng(30).uniform(-math.pi, math.pi, (B, c.n_params))
    out = {'workload': '%d qubits, %d layers (Ry, Rz on every qubit + CX ring), %d parameters, '
                       'batch %d, H = -sum Z_i Z_i+1 - 0.7 sum X_i (open chain)'
                       % (n, layers, c.n_params, B)}
    res = {}
    for name, dt, ck in (('fp32', np.float32, 3 * 3 * n), ('fp64', np.float64, 0)):
        E, G = expectation_and_gradient(c, params[:1], H, dt, ck)  # warm-up
        t0 = time.perf_counter()
        for _ in range(args.adj_steps):
            E, G = expectation_and_gradient(c, params, H, dt, ck)
        dtm = (time.perf_counter() - t0) / args.adj_steps
        res[name] = (E, G)
        out[name + '_grads_per_s'] = B / dtm
        out[name + '_ms_per_batch'] = dtm * 1e3
    out['speedup_fp32_vs_fp64'] = out['fp32_grads_per_s'] / out['fp64_grads_per_s']
    out['max_grad_err_fp32_vs_fp64'] = float(np.max(np.abs(res['fp32'][1] - res['fp64'][1])))
    out['max_energy_err_fp32_vs_fp64'] = float(np.max(np.abs(res['fp32'][0] - res['fp64'][0])))
    out['checkpoint_every_gates_fp32'] = 3 * 3 * n
    return out


def qft_ops(n, seed):
    """QFT without final swaps on |x>, X on qubit i iff rng.random() < 0.5
    (in qubit order): for i: H(q_i), then CU1(pi / 2^(j-i)) controlled by q_j
    on q_i for j > i."""
    rng = np.random.default_rng(seed)
    ops = [('X', (), q, ()) for q in range(n) if rng.random() < 0.5]
    for i in range(n):
        ops.append(('H', (), i, ()))
        for j in range(i + 1, n):
            ops.append(('U1', (math.pi / (1 << (j - i)),), i, (j,)))
    return ops


def run_compiled(args, rt, nat):
    """Per-run latency of whole circuits through the plugin API with one call
    per gate (the reference front-end's pattern; with trace replay, the
    default, a run seen before replays its captured CUDA graph, and without
    it, `per_gate_call_planned_ms`, every run is planned anew), against
    `CompiledCircuit` (the gate table in one call) and its CUDA-graph replay:
    the reference's
    20-qubit QFT case (complex128, and complex64, where the device work is
    small and the host's share shows; X preparation from default_rng(0)) and
    the headline random circuit (complex64).  Wall time from reset to a
    synchronised state, median of the repeats after one warm-up run (which
    plans, and for the graph captures)."""
    from qgate_gb300.circuit import gate_type
    from qgate_gb300.compiled import CompiledCircuit
    out = {}
    cases = [('qft_20q_c128', 20, qft_ops(20, 0), np.float64, 20),
             ('qft_20q_c64', 20, qft_ops(20, 0), np.float32, 20),
             ('random_%dq_c64' % args.qubits, args.qubits, circuit(args.qubits, args.depth),
              np.float32, 3)]
    for label, n, ops, dtype, reps in cases:
        gts = [(gate_type(nm, *a), False, t, list(c)) for nm, a, t, c in ops]
        qs = rt.create_qubit_states(dtype)
        proc = qs.processor
        proc.initialize_qubit_states(qs, n)

        def per_gate():
            proc.reset_qubit_states(qs)
            for gt, adj, t, c in gts:
                if c:
                    proc.apply_controlled_gate(gt, adj, qs, c, t)
                else:
                    proc.apply_gate(gt, adj, qs, t)
            proc.synchronize()

        def median_ms(f):
            f()
            ts = []
            for _ in range(reps):
                t0 = time.perf_counter()
                f()
                ts.append(time.perf_counter() - t0)
            return float(np.median(ts)) * 1e3

        nat.set_trace_replay(False)
        planned = median_ms(per_gate)
        nat.set_trace_replay(True)
        nat.trace_stats(reset=True)
        replayed = median_ms(per_gate)
        st = nat.trace_stats(reset=True)
        res = {'qubits': n, 'gates': len(gts), 'dtype': 'c128' if dtype == np.float64 else 'c64',
               'per_gate_call_ms': replayed, 'per_gate_call_planned_ms': planned,
               'trace_replays': st['hits'], 'trace_captures': st['captures']}
        for graph in (False, True):
            circ = CompiledCircuit(dtype, gts, graph=graph)

            def run():
                proc.reset_qubit_states(qs)
                circ.run(qs)
                proc.synchronize()

            res['graph_replay_ms' if graph else 'compiled_call_ms'] = median_ms(run)
            if graph:
                res['graph_passes'] = circ.stats()[1]
            circ.delete()
        qs.delete()
        out[label] = res
    return out


def run_c4(args, rt, nat):
    """Large single states: a 33-qubit depth-30 random U3+CX circuit
    (default_rng(40)), and a 34-qubit QFT (X preparation from default_rng(41))
    followed by an FP64 sampling pool and 1e8 samples (default_rng(42)), all
    complex64.  The QFT of a basis state has every probability equal to 2^-34,
    so Pr(q = 0) = 1/2 for every qubit and the uniform (k + 1/2) / 2^34 samples
    index k."""
    from qgate_gb300.circuit import gate_type, Lane
    from qgate_gb300 import autotune
    out = {}

    peak, peak_kind = measured_peak_hbm()

    def run(n, ops, label):
        gts = [(gate_type(nm, *a), t, list(c)) for nm, a, t, c in ops]
        qs = rt.create_qubit_states(np.float32)
        proc = qs.processor
        proc.initialize_qubit_states(qs, n)
        proc.synchronize()  # the state's memory allocated outside the timed region
        nat.gate_stats(reset=True)
        nat.timing_all(reset=True)
        nat.timing_enable(True)
        t0 = time.perf_counter()
        # timed from the reset, as in the main step: |0...0> is formed with
        # the circuit's first flush (X gates reaching it first fold into it)
        proc.reset_qubit_states(qs)
        for gt, t, c in gts:
            if c:
                proc.apply_controlled_gate(gt, False, qs, c, t)
            else:
                proc.apply_gate(gt, False, qs, t)
        proc.synchronize()
        dt = time.perf_counter() - t0
        nat.timing_enable(False)
        tm = nat.timing_all(reset=True)
        st = nat.gate_stats(reset=True)
        res = {'qubits': n, 'gates': len(ops), 'passes': st['passes'], 'ms': dt * 1e3,
               'gate_pass_gbs': gate_pass_bytes(n, ops, 8) / dt / 1e9,
               'hbm_gbs_actual': st['bytes'] / dt / 1e9,
               'kernel_ms': {k: v[1] for k, v in tm.items() if v[0]},
               'norm': qs.processor.calc_norm(qs)}
        launches, ms = tm.get('tstage', (0, 0.))
        if launches:
            gbs = 2 * (1 << n) * 8 / (ms / launches / 1e3) / 1e9
            res['tstage'] = {'launches': launches, 'avg_launch_ms': ms / launches, 'gbs': gbs,
                             'frac_of_peak': gbs / peak, 'peak_source': peak_kind}
        out[label] = res
        return qs

    # the 30-qubit circuit's tuned fusion shape (12-lane tensor stages when
    # there is none)
    cached = autotune._load().get(autotune._key(30, np.float32))
    if cached:
        autotune.apply(cached)
    else:
        nat.set_fusion(12)
        nat.set_tensor_blocks(True)
    n1 = args.c4_random_qubits
    if n1 > 0:  # 0 skips it
        ops1 = circuit(n1, 30, seed_angles=40, seed_perm=40)
        qs = run(n1, ops1, 'random_%dq_depth30' % n1)
        qs.delete()
        nat.call('qg_devices_clear')  # return the cached 64 GiB before the 128 GiB state

    n2 = args.c4_qft_qubits
    qs = run(n2, qft_ops(n2, 41), 'qft_%dq' % n2)
    pr = [qs.processor.calc_probability(qs, q) for q in range(n2)]
    out['qft_%dq' % n2]['max_abs_pr0_minus_half'] = float(max(abs(p - 0.5) for p in pr))
    getter = rt.create_qubits_states_getter(np.float32)
    t0 = time.perf_counter()
    pool = getter.create_sampling_pool(list(range(n2)), n2, 0,
                                       [(qs, [Lane(l, l) for l in range(n2)])], [])
    t_pool = time.perf_counter() - t0
    u = np.random.default_rng(42).random(args.c4_samples)
    t0 = time.perf_counter()
    obs = pool.sample(len(u), u)
    t_samp = time.perf_counter() - t0
    N = 1 << n2
    k = np.random.default_rng(43).integers(0, N, 100000)
    mid = pool.sample(len(k), (k + 0.5) / N)
    dev = np.abs(np.asarray(mid.intarray) - k)
    out['pool'] = {'entries': N, 'create_ms': t_pool * 1e3, 'samples': len(u),
                   'sample_ms': t_samp * 1e3, 'samples_per_s': len(u) / t_samp,
                   'midpoint_exact_frac': float(np.mean(dev == 0)),
                   'midpoint_max_index_dev': int(dev.max())}
    pool.delete()
    qs.delete()
    nat.call('qg_devices_clear')
    return out


def run_batch(args, nat):
    """4096 hardware-efficient-ansatz circuits of uneven size (n ~ U{8..20},
    depth ~ U{4..12}, Ry and Rz on every qubit then a CX ladder; default_rng(20)),
    complex64, sum_i <Z_i> per circuit in FP64: circuits per second of the
    call (host planning + one CUDA graph) and of the graph alone, for the one
    persistent launch (default) and for one launch per round, with the bytes
    of the large circuits' stage passes per second."""
    from qgate_gb300.batch import hea_batch, pack, sum_z
    circuits = hea_batch(count=args.batch_circuits, seed=20)
    packed = pack(circuits)
    peak, peak_kind = measured_peak_hbm()
    res = {'workload': '%d circuits, n ~ U{8..20}, depth ~ U{4..12}, Ry+Rz layers + CX ladder, '
                       'sum_i <Z_i> per circuit' % len(circuits),
           'gates': int(packed[1][-1])}
    amps = sum((1 << n) * len(ops) for n, ops in circuits)
    for label, one in (('one_launch', 1), ('per_round_launches', 0)):
        nat.call('qg_set_batch_one_launch', one)
        sum_z(packed=packed)  # warm-up
        nat.timing_all(reset=True)
        nat.gate_stats(reset=True)
        nat.timing_enable(True)
        t0 = time.perf_counter()
        for _ in range(args.batch_steps):
            out = sum_z(packed=packed)
        dt = (time.perf_counter() - t0) / args.batch_steps
        nat.timing_enable(False)
        launches, gms = nat.timing_read('batch', reset=True)
        st = nat.gate_stats(reset=True)
        gms /= max(1, launches)
        stage_bytes = st['bytes'] / args.batch_steps
        res[label] = {'circuits_per_s': len(circuits) / dt, 'ms_per_batch': dt * 1e3,
                      'graph_ms': gms, 'circuits_per_s_graph': len(circuits) / (gms / 1e3),
                      'amplitude_updates_per_s': amps / dt,
                      'stage_passes': st['passes'] / args.batch_steps,
                      'stage_pass_bytes': stage_bytes,
                      'stage_pass_gbs': stage_bytes / (gms / 1e3) / 1e9,
                      'checksum': float(np.sum(out))}
    nat.call('qg_set_batch_one_launch', 1)
    one = res['one_launch']
    res.update({'circuits_per_s': one['circuits_per_s'], 'graph_ms': one['graph_ms'],
                'circuits_per_s_graph': one['circuits_per_s_graph'],
                'bound': 'instruction issue in the tile programs (interpreted register ops '
                         'and shared-memory transposes), not memory: the large circuits\' '
                         'stage passes (read + write of a 64 KB - 8 MB state) move %.0f GB/s, '
                         '%.2f of the %.0f GB/s HBM copy peak (%s); circuits of <= 12 qubits '
                         'never leave shared memory' % (one['stage_pass_gbs'],
                                                        one['stage_pass_gbs'] / peak, peak,
                                                        peak_kind)})
    return res


def observation_kernels(args, rt, nat, proc, qs, n, cs, dtype, Lane, abs2):
    """Per-kernel-class device time and HBM roofline of the observation path
    on the final 2^n state: Pr(lane = 0) (prob), a Pauli expectation (pauli),
    the full probability vector (gather), a sampling pool over all lanes (the
    two-pass fixed-point prefix sum read straight from the state: scan), 1e7
    samples (search) and the |0...0> reset (init).  CUDA events per launch on
    the engine stream; algorithmic bytes = what each kernel must read and
    write once."""
    N = 1 << n
    amp = cs
    getter = rt.create_qubits_states_getter(dtype)
    lanes = [(qs, [Lane(l, l) for l in range(n)])]
    probs = np.empty(N, dtype)
    u = np.random.default_rng(12).random(args.samples)
    # warm the arena and the host buffers once, untimed
    getter.get_states(probs, 0, abs2, lanes, [], N, 0, 1)
    pool = getter.create_sampling_pool(list(range(n)), n, 0, lanes, [])
    pool.sample(args.samples, u)
    pool.delete()
    nat.timing_all(reset=True)
    nat.timing_enable(True)
    proc.calc_probability(qs, 0)
    proc.synchronize()
    nat.timing_enable(False)
    lane0 = nat.timing_all(reset=True).get('prob', (0, 0.))
    nat.timing_enable(True)
    proc.calc_probability(qs, n - 1)
    proc.calc_pauli_expectation(qs, 1 << 3, (1 << 3) | (1 << 7))
    getter.get_states(probs, 0, abs2, lanes, [], N, 0, 1)
    pool = getter.create_sampling_pool(list(range(n)), n, 0, lanes, [])
    pool.sample(args.samples, u)
    pool.delete()
    proc.reset_qubit_states(qs)
    proc.synchronize()
    nat.timing_enable(False)
    tm = nat.timing_all(reset=True)
    peak, kind = measured_peak_hbm()
    # algorithmic bytes per launch (scan: per pool, both passes)
    model = {
        'prob': (N // 2 * amp, 'read the half of the state with the lane at 0 (lane n-1)'),
        'pauli': (N * amp, 'read the state'),
        'gather': (N * amp + N * (amp // 2), 'read the state, write 2^n probabilities'),
        'marginal': (N * amp + N * 8, 'read the state, write 2^n FP64 probabilities'),
        'scan': (2 * N * amp + N * 8,
                 'tile sums read the state; the scan reads it again and writes 2^n 64-bit '
                 'prefix sums'),
        'init': (N * amp, 'write the state'),
    }
    out = {}
    for cls, (launches, ms) in tm.items():
        if not launches:
            continue
        e = {'launches': launches, 'ms': ms}
        per = ms / launches
        if cls == 'scan':
            per = ms  # one pool: its two launches
        if cls in model:
            b, what = model[cls]
            gbs = b / (per / 1e3) / 1e9
            e.update({'algorithmic_bytes': b, 'bytes_are': what, 'gbs': gbs,
                      'frac_of_peak': gbs / peak})
        if cls == 'search':
            e['samples_per_s'] = args.samples / (ms / 1e3)
        out[cls] = e
    if lane0[0]:
        # lanes 0 and 1 split every 32-byte sector: the whole state crosses HBM
        b = N * amp
        gbs = b / (lane0[1] / 1e3) / 1e9
        out['prob_lane0'] = {'launches': lane0[0], 'ms': lane0[1], 'bytes': b,
                             'bytes_are': 'every 32-byte sector of the state (lane 0 splits '
                                          'each sector)',
                             'gbs': gbs, 'frac_of_peak': gbs / peak}
    out['peak_gbs'] = peak
    out['peak_source'] = kind
    return out


def run_e2e(args, rt, nat, qs, step, ops, n, cs, dtype, Lane, abs2):
    """Same metric through the plugin API with host buffers: circuit, full
    probability vector to host, pool + 1e7 samples from host uniforms."""
    getter = rt.create_qubits_states_getter(dtype)
    u = np.random.default_rng(12).random(args.samples)
    probs = np.empty(1 << n, dtype)

    def lane_trans():
        return [(qs, [Lane(l, l) for l in range(n)])]

    def e2e_step():
        step()
        getter.get_states(probs, 0, abs2, lane_trans(), [], 1 << n, 0, 1)
        pool = getter.create_sampling_pool(list(range(n)), n, 0, lane_trans(), [])
        obs = pool.sample(args.samples, u)
        pool.delete()
        return obs

    e2e_step()
    nat.gate_stats(reset=True)
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        e2e_step()
    dt = time.perf_counter() - t0
    stats = nat.gate_stats(reset=True)
    unfused = gate_pass_bytes(n, ops, cs) * args.e2e_steps
    return {'value': unfused / dt / 1e9, 'unit': 'GB/s',
            'h2d_bytes_per_step': args.samples * 8 + len(ops) * 64,
            'd2h_bytes_per_step': (1 << n) * (cs // 2) + args.samples * 8,
            'steps': args.e2e_steps, 'ms_per_step': dt / args.e2e_steps * 1e3,
            'outputs': 'probability vector (2^%d %s) + %d samples' % (
                n, 'float32' if cs == 8 else 'float64', args.samples)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--qubits', type=int, default=30)
    ap.add_argument('--depth', type=int, default=20)
    ap.add_argument('--dtype', default='c64', choices=['c64', 'c128'])
    ap.add_argument('--tile', type=int, default=0,
                    help='fusion tile lanes (0 = autotuned, 1 = fusion off)')
    ap.add_argument('--retune', action='store_true', help='ignore the autotuner cache')
    ap.add_argument('--no-tensor', action='store_true',
                    help='complex64 stages on the CUDA cores (k_rstage) instead of tcgen05 blocks')
    ap.add_argument('--samples', type=int, default=10_000_000)
    ap.add_argument('--e2e-steps', type=int, default=4)
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--no-fidelity', action='store_true',
                    help='skip the complex64-vs-complex128 accuracy check of the final state')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-adjoint', action='store_true')
    ap.add_argument('--no-batch', action='store_true')
    ap.add_argument('--no-compiled', action='store_true')
    ap.add_argument('--no-c4', action='store_true', help='skip the 33/34-qubit large states')
    ap.add_argument('--c4-random-qubits', type=int, default=33, help='0 skips it')
    ap.add_argument('--c4-qft-qubits', type=int, default=34)
    ap.add_argument('--c4-samples', type=int, default=100_000_000)
    ap.add_argument('--batch-circuits', type=int, default=4096)
    ap.add_argument('--batch-steps', type=int, default=3)
    ap.add_argument('--adj-qubits', type=int, default=24)
    ap.add_argument('--adj-batch', type=int, default=64)
    ap.add_argument('--adj-steps', type=int, default=1)
    ap.add_argument('--cpu-seconds', type=float, default=12.0)
    # the reference arm's step: the circuit's first layer at 30 qubits (30 U3
    # + 15 CX), the same gate mix as the whole circuit
    ap.add_argument('--ref-gates', type=int, default=45)
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == 'gb300':
        print('note: fewer than 3 warm-up steps', file=sys.stderr)
    if args.impl == 'reference':
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == '__main__':
    main()
