"""pytest configuration: the `gpu` marker and shared fixtures.

Tests marked gpu run on a GB300 through the C ABI of libpico_gpu.so; the rest
run on any CPU (oracle against golden vectors, host logic, library exports).
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (str(ROOT), str(ROOT / "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libpico_gpu.so")


@pytest.fixture(scope="session")
def oracle():
    import pico_oracle
    pico_oracle.build_oracle()
    return pico_oracle.Oracle()


@pytest.fixture(scope="session")
def ctx():
    import pico_gb300
    from pico_gb300 import build
    build.build()
    c = pico_gb300.Context(0)
    yield c
    c.close()
