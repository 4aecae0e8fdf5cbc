import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "mg-picola-public_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests of the CUDA path")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the oracle and the library once per session (no-ops when fresh)."""
    from oracle import build as ob

    ob.build()
    import build as pb  # mg-picola-public_gb300/build.py

    pb.build()
    yield
