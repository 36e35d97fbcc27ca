"""Minimal stand-ins for the reference front-end's objects that cross the
runtime plugin boundary, for callers that drive the runtime directly
(without `qgate.script` / `qgate.model`).

* `gate_type(name, *args)` — what a runtime reads from a qgate GateType:
  its class name (U, U2, U1, ID, X, Y, Z, H, S, T, RX, RY, RZ, ExpiI, ExpiZ,
  SH; qgate/model/gate_type.py) and `args`.
* `Lane(local, external)` — an entry of a lane transformation
  (qgate/simulator/lanes.py:3-12).
* `null`, `abs2` — the math ops of the states getter
  (qgate/simulator/qubits.py:5-10).
"""

_classes = {}


def gate_type(name, *args):
    cls = _classes.get(name)
    if cls is None:
        cls = type(name, (), {})
        _classes[name] = cls
    g = cls()
    g.args = tuple(args)
    return g


class Lane:
    def __init__(self, local, external):
        self.local = local
        self.external = external


def null(v):
    return v


def abs2(v):
    return v.real ** 2 + v.imag ** 2


prob = abs2
