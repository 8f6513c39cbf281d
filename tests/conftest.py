import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# The reference's shipped input files (synthetic.fil, GBT_Lband_PSR.fil):
# from the PulsarSr tree named by PSR_REFERENCE_DIR, else from the copies
# tests/golden/stage_inputs.py puts in tests/golden/_ref_data/.  Tests that
# need them skip when neither has them.
REFERENCE_DIR = os.environ.get("PSR_REFERENCE_DIR", "")
GOLDEN = os.path.join(ROOT, "tests", "golden")
STAGED = os.path.join(GOLDEN, "_ref_data")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes tens of seconds on CPU")


def reference_file(name: str) -> str:
    for d in (REFERENCE_DIR, STAGED):
        if d and os.path.exists(os.path.join(d, name)):
            return os.path.join(d, name)
    pytest.skip(f"reference input {name} not available")


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
