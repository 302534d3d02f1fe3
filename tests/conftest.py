import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT / "finitevolumemethod.jl_gb300", ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libfvmgpu.so")


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads libfvmgpu.so; fails loudly without a GPU."""
    import fvmgpu
    from fvmgpu import _lib

    fvmgpu.build()
    _lib.load()
    _lib.require_gpu()
    return _lib
