import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if gpu_available():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def engine_lib():
    """Build (if needed) and load libshwfs.so."""
    from dasp_gb300 import build
    build.build()
    from dasp_gb300 import _lib
    return _lib.lib()


@pytest.fixture(scope="session")
def noise_lib():
    from oracle import shwfs_oracle
    return shwfs_oracle.noise_lib()


@pytest.fixture
def rng():
    return np.random.default_rng(1234)
