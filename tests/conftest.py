import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "montecarlox.jl_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmcx_cuda.so")


@pytest.fixture(scope="session")
def mcxlib():
    """Builds (if stale) and loads libmcx_cuda; the device path has no fallback."""
    sys.path.insert(0, PKG)
    import build as mbuild  # montecarlox.jl_gb300/build.py
    mbuild.build()
    import mcx
    mcx._lib.load()
    return mcx


@pytest.fixture(scope="session")
def gpu(mcxlib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return mcxlib
