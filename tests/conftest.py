import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def lib():
    """The built C-ABI library (built in-tree on first use)."""
    import jaxabm_gb300
    jaxabm_gb300.build()
    from jaxabm_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build
    return build.load()


@pytest.fixture(scope="session")
def cuda(lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a visible CUDA device")
    import jaxabm_gb300
    jaxabm_gb300.set_verbose(False)
    return torch.device("cuda", 0)
