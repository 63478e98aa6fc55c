import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available() -> bool:
    try:
        import custen_gb300 as cs
        lib = cs.lib()
        import ctypes
        n = ctypes.c_int(0)
        # cudaGetDeviceCount through the library's runtime: a device synchronize fails without a GPU.
        return lib.custen_device_synchronize() == 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def built():
    """Build the sm_103a library and the C oracles once per session."""
    import custen_gb300 as cs
    import oracle
    cs.build()
    oracle.build()
    return cs


@pytest.fixture(scope="session")
def gpu(built):
    if not gpu_available():
        pytest.fail("GPU test selected but no CUDA device is usable (these tests must run on the GPU box)")
    return built
