import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 host)")
    config.addinivalue_line("markers", "reference: needs the reference source tree to build the harness")


@pytest.fixture(scope="session")
def cuda_lib():
    """The in-tree CUDA library, built on first use."""
    from epic_gb300 import build, load_library
    build.build()
    return load_library()


@pytest.fixture(scope="session")
def gpu(cuda_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a host without a CUDA device")
    return cuda_lib
