import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests" / "golden"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.build_port()
    return O


@pytest.fixture(scope="session")
def af():
    """The library on a GPU.  Fails (does not skip) when the CUDA extension
    is missing, so a GPU run can never pass without the native code."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    import arrayfire_gb300 as A

    A.lib()
    torch.cuda.init()
    A.set_stream(torch.cuda.current_stream())
    return A


@pytest.fixture(scope="session")
def aflib_cpu():
    """The shared library loaded without touching a GPU (symbol checks and
    host-only helpers)."""
    import arrayfire_gb300 as A

    try:
        return A.lib()
    except ImportError:
        from arrayfire_gb300 import build

        build.build()
        return A.lib()
