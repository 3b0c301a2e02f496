import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the CUDA engine")


@pytest.fixture(scope="session")
def engine():
    """The built CUDA engine; GPU tests fail (never skip) if it cannot load."""
    from fast_hdbscan_gb300 import build, _native
    build.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return _native.load()
