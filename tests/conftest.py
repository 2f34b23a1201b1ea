import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "fft3d-fpga_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (a GB300)")


@pytest.fixture(scope="session")
def libpath():
    """Build (incrementally) and return the in-tree libfftfpga.so."""
    sys.path.insert(0, PKG)
    import build as fftgb_build  # fft3d-fpga_gb300/build.py
    return fftgb_build.build()


@pytest.fixture(scope="session")
def lib(libpath):
    from fftgb import _lib
    return _lib.load(libpath)


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def cuda(lib):
    if not gpu_available():
        pytest.fail("GPU test run without a CUDA device")
    import torch
    torch.cuda.init()
    return torch.device("cuda:0")
