import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# The PulsarSr reference tree (read-only).  Only CPU tests that pin the oracle
# against the reference's shipped input files use it; they skip without it.
REFERENCE_DIR = os.environ.get("PSR_REFERENCE_DIR", "/root/reference")
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes tens of seconds on CPU")


def reference_file(name: str) -> str:
    path = os.path.join(REFERENCE_DIR, name)
    if not os.path.exists(path):
        pytest.skip(f"reference input {name} not available")
    return path


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gpu():
    """The libpsr API, after checking that a CUDA device is present."""
    import ctypes
    try:
        cudart = ctypes.CDLL("libcudart.so")
    except OSError:
        import glob
        cands = glob.glob("/usr/local/cuda/lib64/libcudart.so*")
        cudart = ctypes.CDLL(cands[0])
    n = ctypes.c_int(0)
    if cudart.cudaGetDeviceCount(ctypes.byref(n)) != 0 or n.value == 0:
        pytest.fail("no CUDA device: GPU tests need a GB300")
    from pulsarsr_gb300 import build
    build.build()
    import pulsarsr_gb300
    return pulsarsr_gb300
