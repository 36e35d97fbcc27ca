"""The pool's exact integer sampling rule (tests/pool_model.py, what the GPU
pool computes) against the oracle's FP64 pool (the reference's cumsum /
total and upper_bound, qgate/simulator/src/CPUSamplingPool.cpp:16-81): the
same index for every uniform except within rounding of a CDF boundary."""
import numpy as np
import pytest

from oracle import statevec as sv
from tests.pool_model import fixed_point_samples


@pytest.mark.parametrize('kind', ['porter_thomas', 'skewed', 'sparse'])
def test_integer_rule_matches_fp64_pool(kind):
    rng = np.random.default_rng(7)
    n = 1 << 14
    if kind == 'porter_thomas':
        p = rng.exponential(size=n)
    elif kind == 'skewed':
        p = rng.random(n) ** 12
    else:
        p = np.zeros(n)
        p[rng.choice(n, 40, replace=False)] = rng.random(40)
    p = (p / p.sum()).astype(np.float32)
    u = np.concatenate([rng.random(30000), [0., 1. - 2. ** -53]])
    got = fixed_point_samples(p, u)
    want = sv.SamplingPool(p).sample(u)
    # uniforms within the FP64 cumsum's rounding (<= n ulp) of a CDF boundary
    cdf = np.cumsum(p.astype(np.float64)) / float(np.sum(p.astype(np.float64)))
    tau = 4. * n * 2. ** -53
    i = np.searchsorted(cdf, u)
    lo = cdf[np.clip(i - 1, 0, n - 1)]
    hi = cdf[np.clip(i, 0, n - 1)]
    near = (np.abs(u - lo) <= tau) | (np.abs(u - hi) <= tau)
    assert np.array_equal(got[~near], want[~near])
    assert np.mean(near) < 1e-3
    assert np.all(p[got[u < 1.]] > 0)  # zero-probability items are never drawn
