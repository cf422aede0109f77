import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built CUDA library")


@pytest.fixture(scope="session")
def built_lib():
    """Path of the CUDA library, built in-tree if it is missing."""
    from rot2d3c_gb300 import build as b
    return b.build()


@pytest.fixture(scope="session")
def gpu():
    """The CUDA library loaded on a GPU machine; fails loudly otherwise."""
    import torch  # noqa: F401  (only to report the device clearly)
    from rot2d3c_gb300 import build as b
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a visible CUDA device")
    b.build()
    import rot2d3c_gb300 as r
    r.load()
    return r
