import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the library's kernels)")


@pytest.fixture(scope="session")
def oracle():
    from tests.rvtest import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def golden():
    return np.load(ROOT / "tests" / "golden" / "golden.npz")


@pytest.fixture(scope="session")
def rvlib():
    from recview_gb300.build import build_lib
    import recview_gb300
    build_lib()
    return recview_gb300.lib()


@pytest.fixture(scope="session")
def gpu(rvlib):
    """The library with a usable CUDA device; fails (never skips) when none is present."""
    n = rvlib.GetCudaDeviceCount(0)
    assert 0 < n < 0x10000, f"no usable CUDA device (GetCudaDeviceCount -> {n:#x})"
    return rvlib
