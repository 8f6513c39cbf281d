"""PulsarSr search path on GB300 (sm_103a): C ABI in include/psr.h, kernels
in csrc/, and this Python mirror of the reference crate API.

Submodules: fbank, rfi, dedisperse, search, fold, session.  Every compute
call goes through libpsr.so; importing a submodule raises when the library
has not been built (there is no CPU fallback).
"""
from ._lib import (CapacityError, CudaError, DedisperseError, FormatError, InvalidArgument,
                   IoError, PsrError, lib)
from ._lib import TimeoutError_ as WaitTimeout

__all__ = ["PsrError", "FormatError", "IoError", "DedisperseError", "InvalidArgument",
           "CudaError", "CapacityError", "WaitTimeout", "lib", "version"]


def version() -> str:
    return lib().psr_version().decode()
