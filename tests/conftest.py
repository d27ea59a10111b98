import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built libcansgpu.so")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu():
    """The GPU library; a GPU test fails loudly if it is missing or unusable."""
    from utrip_gb300 import capi
    capi.load()
    if not capi.device_ok():
        pytest.fail("no usable sm_103 device: GPU tests must run on a GB300")
    return capi
