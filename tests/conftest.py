import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def mtc():
    """The CUDA library, built in-tree if needed; fails loudly if it cannot load."""
    import mtcheck_gb300
    from mtcheck_gb300 import build
    build.build()
    mtcheck_gb300.load()
    return mtcheck_gb300


@pytest.fixture(scope="session")
def cuda(mtc):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch
