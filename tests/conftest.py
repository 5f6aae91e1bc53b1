import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libedgpu.so")


@pytest.fixture(scope="session")
def eng():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from impuritymodel_gb300 import build

    build()
    from impuritymodel_gb300.engine import get_engine

    return get_engine()
