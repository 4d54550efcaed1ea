import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load the CUDA library; GPU tests fail loudly without it."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu test run without a CUDA device")
    from gammcor_gb300 import build, _lib
    build.build()
    return _lib.load()
