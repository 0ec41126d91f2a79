"""Test configuration: the ``gpu`` marker and import paths.

``-m "not gpu"`` runs on any host (oracle known-answer tests, host logic,
library exports); ``-m gpu`` needs a CUDA device and checks the GPU path
through the C ABI against the oracle.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer-running case")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def aran():
    import aran_gb300 as A
    A.load()
    return A
