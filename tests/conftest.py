import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (HERE, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def cuda_ready():
    """Build the library if needed and require a visible GPU."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu test run without a visible CUDA device")
    from goetia_gb300 import build
    build.build()
    torch.cuda.init()
    return True
