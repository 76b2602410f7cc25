import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gpu_ctx():
    """One gbrt context for the GPU tests; fails loudly if the CUDA library
    or the device is missing (no CPU fallback exists)."""
    from rustracer_gb300 import build, gbrt
    build.build()
    ctx = gbrt.Context(0)
    yield ctx
    ctx.close()
