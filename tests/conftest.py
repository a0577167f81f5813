import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built extension")
    config.addinivalue_line("markers", "slow: longer statistical checks")


@pytest.fixture(scope="session")
def oracle():
    import oracle_py
    oracle_py.build()
    return oracle_py


@pytest.fixture(scope="session")
def native():
    """The built CUDA library; GPU tests fail (not skip) when it is missing."""
    from dtrt_gb300 import build_ext, native as nat
    build_ext.build()
    if nat.device_count() <= 0:
        pytest.fail("no CUDA device visible for a gpu-marked test")
    return nat
