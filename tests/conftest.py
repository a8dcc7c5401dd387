import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")
    config.addinivalue_line("markers", "slow: full-size workloads")


@pytest.fixture(scope="session")
def native_lib():
    """Build (if needed) and load libkazen_gb300.so."""
    from kazen_proto_gb300 import build as kbuild
    kbuild.build()
    from kazen_proto_gb300 import _native
    return _native.lib()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def gpu(native_lib):
    from kazen_proto_gb300 import _native
    if native_lib.kz_device_count() == 0:
        pytest.fail("GPU test collected but no CUDA device is visible")
    return native_lib
