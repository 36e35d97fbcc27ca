"""Autotuner for the fused-stage kernels' tile shape.

The fusion planner packs gates into shared-memory tiles of `tile_lanes`
lanes, run by the register-resident stage kernel with `reg_lanes` lanes per
thread's registers, and closes a stage when its estimated per-amplitude
instruction count passes `cost_budget`; complex64 stages of 12 or 13 lanes
can instead run on the tensor cores as fused 5-lane blocks (`tensor`), with
one or two threads per tile row (`prefetch` = the stage-pipelining switch).  Which shape is fastest
depends on the state size, the precision and the gate mix, so this module
times a candidate grid on a caller-supplied circuit and keeps the best
shape per (device, lanes, precision) in a JSON cache in the user's cache
directory (`$QG_TUNING_CACHE`, else `$XDG_CACHE_HOME/qgate_gb300/tuning.json`,
else `~/.cache/qgate_gb300/tuning.json`), never inside the package.

    from qgate_gb300 import autotune
    best = autotune.tune(n_lanes, np.float32, ops)   # ops: [(name, args, target, controls)]
    autotune.apply(best)
"""
import json
import os
import time

import numpy as np

from . import _native as nat
from .circuit import gate_type



def cache_path():
    """Where tuned shapes are kept (see the module docstring)."""
    p = os.environ.get('QG_TUNING_CACHE')
    if p:
        return p
    base = os.environ.get('XDG_CACHE_HOME') or os.path.join(os.path.expanduser('~'), '.cache')
    return os.path.join(base, 'qgate_gb300', 'tuning.json')


# (tile_lanes, reg_lanes, cost_budget, tensor, prefetch)
CANDIDATES = {
    np.float32: [(10, 4, 0, 0, 0), (11, 4, 0, 0, 0), (11, 5, 0, 0, 0), (12, 4, 0, 0, 0),
                 (12, 5, 0, 0, 0), (13, 4, 0, 0, 0), (13, 5, 0, 0, 0), (12, 4, 130, 0, 0),
                 (11, 4, 130, 0, 0), (12, 5, 0, 1, 0), (12, 5, 0, 1, 1), (13, 5, 0, 1, 0)],
    np.float64: [(10, 4, 0, 0, 0), (11, 4, 0, 0, 0), (12, 4, 0, 0, 0), (13, 4, 0, 0, 0),
                 (11, 3, 0, 0, 0), (12, 3, 0, 0, 0)],
}
# bumped whenever the kernels change in a way that can reorder the candidates
_VERSION = 'v4'


def _norm(c):
    c = tuple(c)
    return c + (0,) * (5 - len(c))


def _key(n_lanes, dtype):
    info = nat.device_info()
    return '%s/%d.%d/%d/%s' % (_VERSION, info['cc_major'], info['cc_minor'], n_lanes,
                               'c128' if dtype == np.float64 else 'c64')


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except Exception:
        return {}


def _save(cache):
    p = cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, 'w') as f:
            json.dump(cache, f, indent=1)
    except OSError:
        pass


def _prec(dtype):
    return nat.PREC_FP64 if dtype == np.float64 else nat.PREC_FP32


def apply(best):
    nat.set_fusion_params(best['prec'], best['tile_lanes'], best['reg_lanes'],
                          best['cost_budget'])
    nat.set_tensor_blocks(best.get('tensor', 0))
    nat.call('qg_set_stage_pipelining', int(best.get('prefetch', 0)))


def _time_candidates(n_lanes, dtype, ops, repeats, cands):
    """[(seconds per run, tile, reg_lanes, budget, tensor, prefetch)] of the
    candidates that apply to this state, on the GPU."""
    from . import gb300runtime as rt
    gts = [(gate_type(nm, *a), t, list(c)) for nm, a, t, c in ops]
    qs = rt.create_qubit_states(dtype)
    proc = qs.processor
    proc.initialize_qubit_states(qs, n_lanes)

    def run():
        proc.reset_qubit_states(qs)
        for gt, t, c in gts:
            if c:
                proc.apply_controlled_gate(gt, False, qs, c, t)
            else:
                proc.apply_gate(gt, False, qs, t)
        proc.synchronize()

    prec = _prec(dtype)
    results = []
    for cand in cands:
        tile, rl, budget, tensor, prefetch = _norm(cand)
        if tile > n_lanes or (tensor and dtype == np.float64):
            continue
        nat.set_fusion_params(prec, tile, rl, budget)
        nat.set_tensor_blocks(tensor)
        nat.call('qg_set_stage_pipelining', prefetch)
        run()
        t0 = time.perf_counter()
        for _ in range(repeats):
            run()
        dt = (time.perf_counter() - t0) / repeats
        results.append((dt, tile, rl, budget, tensor, prefetch))
    qs.delete()
    nat.set_tensor_blocks(0)
    nat.call('qg_set_stage_pipelining', 0)
    return results


def tune(n_lanes, dtype, ops, repeats=2, use_cache=True, candidates=None):
    """Times every candidate shape on `ops` applied to a resident 2^n_lanes
    state and returns the fastest as a dict (also cached on disk, keyed by
    the kernels' version, the device's compute capability, the lane count and
    the precision; an explicit `candidates` list is timed but not cached).
    The chosen shape is applied."""
    key = _key(n_lanes, dtype)
    cache = _load()
    if use_cache and key in cache and candidates is None:
        apply(cache[key])
        return cache[key]
    results = sorted(_time_candidates(n_lanes, dtype, ops, repeats,
                                      candidates or CANDIDATES[dtype]))
    if not results:
        raise ValueError('no candidate shape fits a %d-lane state.' % n_lanes)
    dt, tile, rl, budget, tensor, prefetch = results[0]
    best = {'prec': _prec(dtype), 'tile_lanes': tile, 'reg_lanes': rl, 'cost_budget': budget,
            'tensor': tensor, 'prefetch': prefetch, 'circuit_ms': dt * 1e3,
            'table': [list(r[1:]) + [r[0] * 1e3] for r in results]}
    if candidates is None:
        cache[key] = best
        _save(cache)
    apply(best)
    return best
