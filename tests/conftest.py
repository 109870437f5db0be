import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device (runs through libsyfrack_gpu.so)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle  # tests/conftest puts oracle/ on the path

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_ctx():
    from syfrack_gb300 import GpuContext

    ctx = GpuContext()
    yield ctx
    ctx.close()


@pytest.fixture(scope="session")
def renderer(gpu_ctx):
    from syfrack_gb300 import Renderer

    return Renderer(gpu_ctx)
