"""The autotuner's selection and cache on the CPU (qgate_gb300/autotune.py):
the timing of candidates on the GPU is replaced by fixed numbers, so what is
checked is the choice of the fastest shape, the cache key (kernel version,
compute capability, lanes, precision), the cache's location outside the
package, reuse of a cached entry without timing, re-timing with
use_cache=False, and that explicit candidate lists are not cached."""
import json
import os

import numpy as np
import pytest

from qgate_gb300 import autotune


@pytest.fixture
def tuner(tmp_path, monkeypatch):
    path = tmp_path / 'tune' / 'tuning.json'
    monkeypatch.setenv('QG_TUNING_CACHE', str(path))
    calls = {'timed': 0, 'applied': []}

    def fake_time(n, dtype, ops, repeats, cands):
        calls['timed'] += 1
        # in this fake a run takes (tile - 5 * tensor) ms: the 12-lane tensor
        # shapes are fastest, the one-thread-per-row variant first on ties
        return [(1e-3 * (c[0] - 5 * c[3]), *autotune._norm(c)[:5]) for c in cands
                if c[0] <= n]

    monkeypatch.setattr(autotune, '_time_candidates', fake_time)
    monkeypatch.setattr(autotune, '_key', lambda n, dt: '%s/10.3/%d/%s' % (
        autotune._VERSION, n, 'c128' if dt == np.float64 else 'c64'))
    monkeypatch.setattr(autotune, 'apply', lambda best: calls['applied'].append(best))
    return path, calls


def test_cache_lives_outside_the_package(tmp_path, monkeypatch):
    pkg = os.path.dirname(os.path.abspath(autotune.__file__))
    monkeypatch.delenv('QG_TUNING_CACHE', raising=False)
    monkeypatch.setenv('XDG_CACHE_HOME', str(tmp_path))
    assert autotune.cache_path() == str(tmp_path / 'qgate_gb300' / 'tuning.json')
    monkeypatch.delenv('XDG_CACHE_HOME')
    assert not autotune.cache_path().startswith(pkg)


def test_picks_the_fastest_and_caches_it(tuner):
    path, calls = tuner
    best = autotune.tune(20, np.float32, [])
    assert (best['tile_lanes'], best['tensor'], best['prefetch']) == (12, 1, 0)
    assert calls['timed'] == 1 and calls['applied'] == [best]
    stored = json.loads(path.read_text())
    key = '%s/10.3/20/c64' % autotune._VERSION
    assert stored[key]['tile_lanes'] == best['tile_lanes']
    # cached: no timing, the stored shape is applied
    again = autotune.tune(20, np.float32, [])
    assert calls['timed'] == 1 and again == stored[key] and calls['applied'][-1] == again
    # use_cache=False times again; complex128 has its own entry
    autotune.tune(20, np.float32, [], use_cache=False)
    autotune.tune(20, np.float64, [])
    assert calls['timed'] == 3
    assert set(json.loads(path.read_text())) == {key, '%s/10.3/20/c128' % autotune._VERSION}


def test_explicit_candidates_are_timed_not_cached(tuner):
    path, calls = tuner
    best = autotune.tune(11, np.float32, [], candidates=[(11, 4, 0, 0, 0), (10, 4, 0, 0, 0)])
    assert best['tile_lanes'] == 10 and calls['timed'] == 1
    assert not path.exists()
    with pytest.raises(ValueError, match='no candidate'):
        autotune.tune(8, np.float32, [], candidates=[(12, 4, 0, 0, 0)])
