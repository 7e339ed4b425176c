import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def built():
    """Build the native library and the CPU checkers once per session."""
    from contour3d_gb300 import build as b
    from oracle import lib as olib
    b.build()
    olib.build(with_reference=False)
    return True


@pytest.fixture(scope="session")
def oracle(built):
    from oracle.lib import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def gpu(built):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a GPU test ran without a visible CUDA device")
    from contour3d_gb300 import lib
    return lib.load()
