"""psr_raw_power_noalloc (fixed device scratch, no allocation) against
psr_raw_power, through the C ABI.

The file name sorts last so the GPU test also runs after every other test in
the same process; it passes alone in a fresh process too.  The tolerance is
the one of the raw-power parity tests: bit-exact.
"""
import ctypes as C

import numpy as np
import pytest

MAX_LEN = 1 << 20  # PSR_RAW_POWER_NOALLOC_MAX_LEN


def _entry():
    from pulsarsr_gb300 import _lib
    f = _lib.lib().psr_raw_power_noalloc
    f.argtypes = [C.POINTER(C.c_float), C.c_uint64, C.POINTER(C.c_float), C.c_void_p]
    f.restype = C.c_int
    return f


def noalloc_power(series, stream=None):
    from pulsarsr_gb300 import _lib
    s = np.ascontiguousarray(series, dtype=np.float32)
    n = 2 * (1 << (s.size - 1).bit_length())
    out = np.full(n // 2 + 1, np.nan, dtype=np.float32)
    _lib.check(_entry()(s.ctypes.data_as(C.POINTER(C.c_float)), s.size,
                        out.ctypes.data_as(C.POINTER(C.c_float)), stream))
    return out


def test_noalloc_rejects_series_above_maximum():
    """The size check runs before any CUDA call, so it needs no GPU."""
    from pulsarsr_gb300 import CapacityError, build
    build.build()
    s = np.zeros(MAX_LEN + 1, dtype=np.float32)
    with pytest.raises(CapacityError, match="fixed scratch maximum of 1048576 samples"):
        noalloc_power(s)


def _cudart():
    try:
        return C.CDLL("libcudart.so")
    except OSError:
        import glob
        return C.CDLL(sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*"))[0])


@pytest.mark.gpu
def test_noalloc_matches_raw_power_twice_in_a_row(gpu):
    from pulsarsr_gb300 import search
    rng = np.random.default_rng(2026)
    # Single-CTA FFT sizes, four-step sizes, the 531000-sample series of the
    # 96-channel 4-bit search and the maximum; the sizes alternate, so the
    # twiddle tables held in the scratch are rebuilt between calls.
    for n in (1000, 300_000, 4097, 531_000, MAX_LEN, 2):
        for s in (rng.normal(0, 1, n).astype(np.float32),
                  np.rint(rng.normal(800, 30, n)).astype(np.float32)):
            want = search.raw_power(s)
            first = noalloc_power(s)
            second = noalloc_power(s)
            assert first.tobytes() == want.tobytes(), n
            assert second.tobytes() == want.tobytes(), n


@pytest.mark.gpu
def test_noalloc_on_a_caller_stream(gpu):
    from pulsarsr_gb300 import search
    rt = _cudart()
    st = C.c_void_p()
    assert rt.cudaStreamCreateWithFlags(C.byref(st), C.c_uint(1)) == 0  # non-blocking
    try:
        s = np.rint(np.random.default_rng(7).normal(50, 5, 263_500)).astype(np.float32)
        want = search.raw_power(s)
        assert noalloc_power(s, st).tobytes() == want.tobytes()
        assert noalloc_power(s, st).tobytes() == want.tobytes()
    finally:
        rt.cudaStreamDestroy(st)


@pytest.mark.gpu
def test_noalloc_allocates_no_device_memory(gpu):
    """After warm-up calls of every size (which load the modules and their
    kernels, and so reserve the fixed array), further calls of changing sizes
    leave the device's free memory unchanged."""
    rt = _cudart()
    rng = np.random.default_rng(11)
    series = [rng.normal(0, 1, n).astype(np.float32) for n in (1000, 300_000, 4097, MAX_LEN, 2)]
    for s in series:
        noalloc_power(s)
    free0, free1, total = C.c_size_t(), C.c_size_t(), C.c_size_t()
    assert rt.cudaDeviceSynchronize() == 0
    assert rt.cudaMemGetInfo(C.byref(free0), C.byref(total)) == 0
    for s in series + series[::-1]:
        noalloc_power(s)
    assert rt.cudaDeviceSynchronize() == 0
    assert rt.cudaMemGetInfo(C.byref(free1), C.byref(total)) == 0
    assert free1.value == free0.value
