import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (ROOT, HERE, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA library through its C-ABI)")


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle (built on first use)."""
    import pyoracle as po
    po.build()
    return po


@pytest.fixture(scope="session")
def cntc():
    """The GB300 library, loaded through its C-ABI.  GPU tests fail (not skip) without a GPU:
    the library has no CPU path."""
    import torch
    import contact_gb300 as cg
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    cg.load()
    return cg
