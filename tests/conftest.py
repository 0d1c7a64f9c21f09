import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cnn-crf-stereo_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the library's kernels")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def cuda():
    """The GPU tests must run on a GPU: no silent skip, no fallback."""
    import torch
    assert torch.cuda.is_available(), "GPU test collected on a machine without CUDA"
    import cnncrf
    cnncrf.lib()  # raises if libcnncrf.so is missing
    return torch
