import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libhg_gpu.so)")


@pytest.fixture(scope="session")
def ctx():
    """A libhg_gpu context on device 0 (GPU tests only; no CPU fallback)."""
    import libhybridgrains_gb300 as hg
    from libhybridgrains_gb300 import build
    build.build()
    c = hg.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def golden_dir():
    return os.path.join(ROOT, "tests", "golden")
