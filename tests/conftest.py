import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300) and the built libngg.so')


@pytest.fixture(scope='session')
def ngg():
    """The built library (compiled on first use); GPU tests only."""
    from cngi_prototype_gb300 import build, _lib
    build.build()
    _lib.load()
    return _lib


def load_golden(name):
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, name + '.npz')))
