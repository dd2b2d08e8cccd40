import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.lib()
    return o


@pytest.fixture(scope="session")
def cuda():
    import torch
    # GPU tests run only when selected (-m gpu); without a device they fail
    # rather than skip, so that a box without a usable GPU cannot pass them.
    assert torch.cuda.is_available(), "GPU test selected but no CUDA device is available"
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def F(cuda):
    from tucuda_gb300 import filters
    filters._lib.load()
    return filters
