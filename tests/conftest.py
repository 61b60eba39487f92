import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libfdtd_gb300.so")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture
def fd():
    """The GB300 package with its backend reset to float64 after the test."""
    import fdtd_gb300

    yield fdtd_gb300
    fdtd_gb300.set_backend("gb300.float64")
