"""Sample containers returned by the sampling pool.

When the reference front-end (`qgate`) is importable, its own
`ObservationList` is used so that results are indistinguishable from the
reference runtimes' (qgate/simulator/native_sampling_pool.py:19-24).
Otherwise this module provides containers with the same constructors and
behaviour (qgate/simulator/observation.py:8-127): `ObservationList` with
`intarray`, `len()`, indexing (an `Observation` per item, an
`ObservationList` per slice), iteration, `obs(ref)` bit extraction with `None`
for empty (never-used) qregs and `histgram()` (an `ObservationHistgram`);
`Observation` with `int`, `int()` and `obs(ref)`, comparable only with another
`Observation`.  Iteration yields `Observation`s (the reference's iterator is
constructed with one argument too few and cannot run).
"""
import collections
import numbers

try:  # the reference front-end, when installed
    from qgate.simulator.observation import (  # noqa: F401
        Observation, ObservationHistgram, ObservationList)
except Exception:  # pragma: no cover - depends on the environment

    def _bit_of(reflist, ref):
        if ref not in reflist:
            raise RuntimeError('unknown ref, {}.'.format(ref))
        return 1 << reflist.index(ref)

    class Observation:
        """One sample: its integer value (bit j = qreg reflist[j]); bits of
        never-used qregs read as None."""

        def __init__(self, reflist, value, none_mask):
            self._reflist = reflist
            self._value = value
            self._none_mask = none_mask

        def __int__(self):
            return int(self._value)

        @property
        def int(self):
            return self._value

        def __call__(self, ref):
            bit = _bit_of(self._reflist, ref)
            if self._value & bit:
                return 1
            return None if self._none_mask & bit else 0

        def _check(self, other):
            if isinstance(other, numbers.Integral):
                raise ValueError('To compare with integer, use int() or Observation.int property.')

        def __eq__(self, other):
            self._check(other)
            if not isinstance(other, Observation):
                raise TypeError('comparison with Observation and {} not supported.'
                                .format(type(other)))
            return (self._reflist == other._reflist and self._value == other._value
                    and self._none_mask == other._none_mask)

        def __ne__(self, other):
            return not self.__eq__(other)

        def __lt__(self, other):
            self._check(other)
            return NotImplemented

        __hash__ = None

    class ObservationHistgram:
        """Counts of sampled values: `hist[value]` (0 if never drawn),
        `n_samples`, and the dict views."""

        def __init__(self, hist, n_bits, n_samples):
            self._hist = hist
            self._n_bits = n_bits
            self._n_samples = n_samples

        @property
        def n_samples(self):
            return self._n_samples

        def __len__(self):
            return len(self._hist)

        def __iter__(self):
            return iter(self._hist)

        def __getitem__(self, key):
            return self._hist.get(key, 0)

        def keys(self):
            return self._hist.keys()

        def values(self):
            return self._hist.values()

        def items(self):
            return self._hist.items()

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
            return Observation(self._reflist, self._values[key], self._mask)

        def __iter__(self):
            for v in self._values:
                yield Observation(self._reflist, v, self._mask)

        def __call__(self, ref):
            bit = _bit_of(self._reflist, ref)
            if self._mask & bit:
                return [None] * len(self._values)
            return [1 if (int(v) & bit) else 0 for v in self._values]

        def histgram(self):
            hist = collections.Counter(int(v) for v in self._values)
            return ObservationHistgram(hist, len(self._reflist), len(self))
