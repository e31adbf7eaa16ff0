import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def gpu():
    """One GPU context for the session; the native library must load."""
    from tracer_gb300.native import GpuContext
    ctx = GpuContext(0)
    yield ctx
    ctx.close()
