import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300, sm_103a)')


@pytest.fixture(scope='session')
def rt():
    """The GB300 runtime module; GPU tests only.  Fails (never skips) when the
    library is missing, so a missing build cannot pass silently."""
    from qgate_gb300 import gb300runtime
    return gb300runtime
