import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built library")


@pytest.fixture(scope="session")
def cuda_lib():
    """The built CUDA library on a CUDA device; GPU tests fail loudly without it."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    from botorch_gb300 import _native

    return _native.lib()
