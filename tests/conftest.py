import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C-ABI")


@pytest.fixture(scope="session")
def engine():
    """The engine library, built in-tree; GPU tests fail loudly if it cannot load."""
    from seqan_gb300 import _native
    _native.build()
    return _native.default_context()
