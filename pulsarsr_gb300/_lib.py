"""ctypes binding of libpsr.so (the C ABI declared in include/psr.h).

The library is loaded from pulsarsr_gb300/_build/ (built in-tree by
pulsarsr_gb300/build.py).  There is no fallback: if the library is missing
or fails to load, importing the API raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpsr.so")

PSR_OK, PSR_EIO, PSR_EFORMAT, PSR_EDEDISPERSE, PSR_EINVAL, PSR_ECUDA, PSR_ETIMEOUT, \
    PSR_ECAPACITY = range(8)


class PsrError(RuntimeError):
    """Base class; .code is the C status."""

    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


class IoError(PsrError):
    pass


class FormatError(PsrError):
    pass


class DedisperseError(PsrError):
    pass


class InvalidArgument(PsrError):
    pass


class CudaError(PsrError):
    pass


class TimeoutError_(PsrError):
    pass


class CapacityError(PsrError):
    pass


_ERRORS = {PSR_EIO: IoError, PSR_EFORMAT: FormatError, PSR_EDEDISPERSE: DedisperseError,
           PSR_EINVAL: InvalidArgument, PSR_ECUDA: CudaError, PSR_ETIMEOUT: TimeoutError_,
           PSR_ECAPACITY: CapacityError}


class Header(C.Structure):
    _fields_ = [("nchans", C.c_int64), ("nbits", C.c_int64), ("tsamp", C.c_double),
                ("fch1", C.c_double), ("foff", C.c_double), ("data_offset", C.c_int64)]


class Candidate(C.Structure):
    _fields_ = [("frequency_hz", C.c_double), ("period_s", C.c_double), ("dm", C.c_double),
                ("harmonics", C.c_uint64), ("score", C.c_double)]


class SearchConfig(C.Structure):
    _fields_ = [("min_hz", C.c_double), ("max_hz", C.c_double), ("threshold", C.c_double),
                ("max_candidates", C.c_uint64), ("birdies", C.POINTER(C.c_double)),
                ("nbirdies", C.c_uint64), ("max_harmonics", C.c_uint64)]


class ProfileStats(C.Structure):
    _fields_ = [("period_s", C.c_double), ("snr", C.c_double),
                ("reduced_chi_square", C.c_double)]


class Measurement(C.Structure):
    _fields_ = [("snr", C.c_double), ("on_samples", C.c_uint64), ("off_samples", C.c_uint64),
                ("mean_difference", C.c_double), ("standard_error", C.c_double)]


_lib: C.CDLL | None = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is not built; run pulsarsr_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        L.psr_version.restype = C.c_char_p
        L.psr_last_error.restype = C.c_uint64
        L.psr_session_payload_device.restype = C.c_void_p
        L.psr_session_stream.restype = C.c_void_p
        L.psr_session_payload_device.argtypes = [C.c_void_p]
        L.psr_session_stream.argtypes = [C.c_void_p]
        L.psr_session_free.argtypes = [C.c_void_p]
        L.psr_fb_free.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def last_error() -> str:
    L = lib()
    buf = C.create_string_buffer(4096)
    L.psr_last_error(buf, C.c_uint64(len(buf)))
    return buf.value.decode(errors="replace")


def check(rc: int) -> None:
    if rc != PSR_OK:
        raise _ERRORS.get(rc, PsrError)(rc, last_error())
