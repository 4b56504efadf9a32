import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def lib():
    import gputools_gb300 as g
    g.build()
    return g.load()


@pytest.fixture(scope="session")
def gpu(lib):
    """The library, on a machine with a CUDA device (fails loudly otherwise)."""
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return lib


@pytest.fixture
def rng():
    return np.random.default_rng(12345)
