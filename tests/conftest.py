import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a Blackwell (sm_103) GPU and the built CUDA library")


@pytest.fixture(scope="session")
def ddla():
    """The product library, built in-tree (no fallback: a build failure fails the test)."""
    from ddla_gb300 import build
    build.build()
    import ddla_gb300
    ddla_gb300.lib()
    return ddla_gb300


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.lib()
    return oracle
