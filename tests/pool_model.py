"""The sampling pool's rule on exact integers, for the tests: each
probability p becomes q = round(p * 2^60) (to nearest, ties to even; exact in
float64 for float32 and float64 p), P = prefix sums of q, and a uniform u
selects the first i with P[i] > floor(u * P[-1]), clamped to n - 1; negative
and NaN u select 0.  This is the reference's upper_bound over its normalised
CDF (qgate/simulator/src/CPUSamplingPool.cpp:16-49, 71-81) evaluated without
rounding."""
import numpy as np


def fixed_point_samples(probs, u):
    q = np.rint(np.asarray(probs).astype(np.float64) * 2.0 ** 60).astype(np.uint64)
    P = np.cumsum(q, dtype=np.uint64)
    T = int(P[-1])
    out = np.zeros(len(u), np.int64)
    for k, v in enumerate(np.asarray(u, np.float64)):
        if not v >= 0.:
            continue
        if v >= 1.:
            out[k] = len(P) - 1
            continue
        num, den = abs(float(v)).as_integer_ratio()
        t = (num * T) // den
        out[k] = min(int(np.searchsorted(P, np.uint64(t), side='right')), len(P) - 1)
    return out
