import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built native library")


@pytest.fixture(scope="session")
def oracle():
    import accfft_oracle

    accfft_oracle.build()
    return accfft_oracle


@pytest.fixture(scope="session")
def native():
    """The product library; built once per session if missing."""
    import accfft_gb300
    from accfft_gb300 import build

    if not os.path.exists(accfft_gb300.LIB_PATH):
        build.build()
    accfft_gb300.lib()
    return accfft_gb300


@pytest.fixture(scope="session")
def cuda(native):
    import torch

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    torch.cuda.init()
    return torch


def rng(seed=0):
    return np.random.default_rng(seed)
