"""Sample containers returned by the sampling pool.

When the reference front-end (`qgate`) is importable, its own
`ObservationList` is used so that results are indistinguishable from the
reference runtimes' (qgate/simulator/native_sampling_pool.py:19-24).
Otherwise this module provides a container with the same constructor and the
accessors the sampling API relies on (qgate/simulator/observation.py:53-100):
`intarray`, `len()`, indexing, `obs(ref)` bit extraction with `None` for
empty (never-used) qregs, and `histgram()`.
"""
import collections

try:  # the reference front-end, when installed
    from qgate.simulator.observation import ObservationList  # noqa: F401
except Exception:  # pragma: no cover - depends on the environment

    class ObservationList:
        def __init__(self, reflist, values, mask):
            self._reflist = reflist
            self._values = values
            self._mask = mask

        @property
        def intarray(self):
            return self._values

        def __len__(self):
            return len(self._values)

        def __getitem__(self, key):
            if isinstance(key, slice):
                return ObservationList(self._reflist, self._values[key], self._mask)
            return int(self._values[key])

        def __call__(self, ref):
            if ref not in self._reflist:
                raise RuntimeError('unknown ref, {}.'.format(ref))
            bit = 1 << self._reflist.index(ref)
            if self._mask & bit:
                return [None] * len(self._values)
            return [1 if (int(v) & bit) else 0 for v in self._values]

        def histgram(self):
            return collections.Counter(int(v) for v in self._values)
