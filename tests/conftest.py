"""Shared test setup: import paths, the `gpu` marker, library fixtures.

CPU tests (-m "not gpu") cover the oracle, its agreement with the reference's
recorded outputs (tests/golden), host-side logic and the C ABI's exported
symbols.  GPU tests call the CUDA library through its C ABI and compare with
the oracle on the same seeded inputs.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "surface-remesher_gb300")
for p in (os.path.join(PKG, "python"), os.path.join(ROOT, "oracle"), PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc
    orc.lib()
    return orc


@pytest.fixture(scope="session")
def gcvt_lib():
    """The CUDA library; building it first if this checkout has no build."""
    import gcvt_gb300
    if not os.path.exists(gcvt_gb300.LIB_PATH):
        import build
        build.build()
    return gcvt_gb300


@pytest.fixture(scope="session")
def cuda_device():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a visible CUDA device")
    return torch.device("cuda:0")
