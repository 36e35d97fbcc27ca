"""qgate_gb300 — GB300-native (sm_103a) state-vector engine behind qgate's
runtime plugin protocol.

* `qgate_gb300.gb300runtime` is a runtime module ("defpkg") for the reference
  front-end's `Simulator(defpkg, **prefs)`; `simulator(**prefs)` builds one
  when the `qgate` front-end is importable.
* The engine itself is libqgate_gb300.so (C ABI: include/qgate_gb300.h),
  loaded by `qgate_gb300._native`; importing that module (or anything that
  uses the engine) fails loudly if the library has not been built.
* `qgate_gb300.csrc.build` builds the library in-tree.
* Beyond the runtime protocol: `compiled` (a gate table applied in one call,
  CUDA-graph replay), `qasm` (OpenQASM 2.0 programs lowered to compiled
  circuits), `adjoint` (batched adjoint gradients), `batch` (many small
  circuits in one persistent launch), `autotune` (fused-stage shapes).
"""

__all__ = ['simulator']


def simulator(**prefs):
    """`qgate.simulator.cuda(**prefs)` with the GB300 runtime
    (qgate/simulator/__init__.py:26-28)."""
    from qgate.simulator.simulator import Simulator
    from . import gb300runtime
    return Simulator(gb300runtime, **prefs)
