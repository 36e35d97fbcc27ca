"""Imports the reference qgate 0.2.2 package (front-end + its own C++ CPU runtime).

Test infrastructure only.  Used by the golden-fixture generator to run the
reference itself; never imported by the product, the GPU tests, smoke() or
bench.py (the reference sources are not present where those run).

* The reference's `qgate/__init__.py:4` imports `qgate.openqasm`, which needs
  the absent `ply` package (`qgate/openqasm/lex.py:1`); it is stubbed here.
* Its `glue` / `cpuext` extensions (`qgate/simulator/cpuruntime.py:1`,
  `qgate/simulator/cpumatrix.py:2`) are the ones `oracle/Makefile` compiled
  into `oracle/_ref/`; they are registered under their package names before
  `qgate.simulator` is imported.
"""
import glob
import importlib.util
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))

# Where the reference's sources are mounted in the build container; the
# QGATE_REF_ROOT environment variable overrides it.  Only the scripts that
# read the reference itself (the fixture generators, the oracle's reference
# build) use it.
DEFAULT_REF_ROOT = '/root/reference'


def reference_root():
    return os.environ.get('QGATE_REF_ROOT', DEFAULT_REF_ROOT)


def import_reference(ref_root=None):
    ref_root = ref_root or reference_root()
    if 'qgate' in sys.modules and hasattr(sys.modules['qgate'], 'simulator'):
        return sys.modules['qgate']
    if not os.path.isdir(os.path.join(ref_root, 'qgate')):
        raise RuntimeError('reference sources not found at %s' % ref_root)
    sys.modules.setdefault('qgate.openqasm', types.ModuleType('qgate.openqasm'))
    for name in ('glue', 'cpuext'):
        paths = glob.glob(os.path.join(HERE, '_ref', name + '*.so'))
        if not paths:
            raise RuntimeError('oracle/_ref/%s not built: run make -C oracle ref' % name)
        full = 'qgate.simulator.' + name
        spec = importlib.util.spec_from_file_location(full, paths[0])
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        sys.modules[full] = mod
    if ref_root not in sys.path:
        sys.path.insert(0, ref_root)
    import qgate  # noqa: E402
    return qgate
