"""rfi: exact median and block-statistics masking on the GPU.

Mirrors rfi::{median, mask} (rfi/src/lib.rs:4-96).  mask() modifies the
device samples of a Filterbank in place, exactly as the reference modifies
its array.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from ._lib import check, lib
from .fbank import Filterbank


@dataclass
class Mask:
    channels: list = field(default_factory=list)
    blocks: list = field(default_factory=list)
    block_samples: int = 0
    masked_fraction: float = 0.0


def median(values) -> float:
    v = np.ascontiguousarray(values, dtype=np.float32)
    out = C.c_float()
    check(lib().psr_median(v.ctypes.data_as(C.POINTER(C.c_float)), C.c_uint64(v.size),
                           C.byref(out)))
    return float(out.value)


def mask(fb: Filterbank, block_samples: int, threshold: float) -> Mask:
    nch = fb.header.nchans
    nb = -(-fb.nsamples // block_samples)
    ch = np.zeros(nch, dtype=np.uint64)
    bl = np.zeros(max(nb, 1), dtype=np.uint64)
    nc, nbb, frac = C.c_uint64(), C.c_uint64(), C.c_double()
    check(lib().psr_rfi_mask(fb.handle, C.c_uint64(block_samples), C.c_float(threshold),
                             ch.ctypes.data_as(C.POINTER(C.c_uint64)), C.byref(nc),
                             bl.ctypes.data_as(C.POINTER(C.c_uint64)), C.c_uint64(bl.size),
                             C.byref(nbb), C.byref(frac)))
    return Mask([int(x) for x in ch[:nc.value]], [int(x) for x in bl[:nbb.value]],
                int(block_samples), float(frac.value))


def channel_stats(fb: Filterbank):
    """The per-channel (means, variances) rfi::mask computes
    (rfi/src/lib.rs:35-43), bit for bit; the filterbank is not modified."""
    nch = fb.header.nchans
    m = np.zeros(nch, dtype=np.float32)
    v = np.zeros(nch, dtype=np.float32)
    check(lib().psr_channel_stats(fb.handle, m.ctypes.data_as(C.POINTER(C.c_float)),
                                  v.ctypes.data_as(C.POINTER(C.c_float))))
    return m, v
