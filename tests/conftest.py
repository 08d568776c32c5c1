import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def built():
    """Build the oracle and the CUDA library in-tree (no-op when up to date)."""
    from oracle.build_oracle import build_oracle
    from phyloacc_gb300.build import build

    build_oracle()
    build()
    return True
