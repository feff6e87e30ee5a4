import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on a GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    """Make sure libtmcore.so and the oracle exist (nvcc/gcc build, no GPU needed)."""
    import oracle
    from torchmorph_gb300 import _build

    _build.build()
    oracle.build()
    yield


@pytest.fixture
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("CUDA device required")
    return torch.device("cuda:0")
