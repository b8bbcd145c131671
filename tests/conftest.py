import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

PKG = "2018_dictionary_tomography_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "slow: long-running test")


@pytest.fixture(scope="session")
def gr():
    return importlib.import_module(PKG)


@pytest.fixture(scope="session")
def eng():
    return importlib.import_module(PKG + ".engine")


@pytest.fixture(scope="session")
def cuda_ready():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return True
