"""Shared fixtures.  `gpu` marks tests that need a GB300 (they call the CUDA library through the
C-ABI); everything else runs on the CPU (oracle, host logic, symbol checks)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lib():
    import gsstructuralanalysis_gb300 as G
    from gsstructuralanalysis_gb300 import build as B
    B.build()
    return G.load_library()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build_oracle()
    return oracle
