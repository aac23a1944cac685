import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Build the CUDA library and the CPU oracle once per session."""
    from parallellbmcranfield_gb300 import build as B
    from oracle import oracle as O

    B.build()
    O.build()
    return True
