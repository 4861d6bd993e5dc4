import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the native kernels)")


@pytest.fixture(scope="session")
def lib():
    """The built C-ABI library (compiled on first use; never a Python fallback)."""
    from cumf_sgd_gb300 import build, _lib
    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.build_oracle()
    return oracle


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


GOLDEN = os.path.join(ROOT, "tests", "golden")
