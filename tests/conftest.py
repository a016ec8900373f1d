"""Shared test set-up: the `gpu` marker, native builds, and the CPU oracle."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (CUDA device)")


@pytest.fixture(scope="session")
def native():
    import cpvulkan_gb300 as c
    c.build()
    return c


@pytest.fixture(scope="session")
def oracle():
    from tests import oracle_binding
    return oracle_binding.load()


@pytest.fixture(scope="session")
def gpu_ctx(native):
    if not native.device_available():
        pytest.fail("a gpu-marked test ran without a usable CUDA device")
    ctx = native.Context()
    yield ctx
    ctx.close()
