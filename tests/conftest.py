import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and runs through libprothgpu")
    config.addinivalue_line("markers", "slow: long-running CPU check")


@pytest.fixture(scope="session")
def gmp():
    from tests import _gmp
    if not _gmp.available():
        pytest.skip("libgmp.so.10 not available")
    return _gmp


@pytest.fixture(scope="session")
def oracle():
    from tests import _oracle
    _oracle.lib()
    return _oracle
