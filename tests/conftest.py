import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built backend library")


@pytest.fixture(scope="session")
def oracle():
    from stwo_gb300.build import build_oracle

    build_oracle()
    import oracle.pyoracle as O

    return O


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from stwo_gb300.build import build_backend

    build_backend()
    from stwo_gb300 import _lib

    _lib.call("stwo_device_init", 0)
    from stwo_gb300.backend import CudaBackend

    return CudaBackend
