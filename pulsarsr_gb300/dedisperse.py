"""dedisperse: FP64 delay tables and GPU incoherent dedispersion.

Mirrors dedisperse::{delays, dm_step, plan, apply} (dedisperse/src/lib.rs:
9-90).  apply() takes a device Filterbank; apply_trials() runs many trial
DMs in one launch (the CLI trial loop without the periodicity step).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, lib
from .fbank import Filterbank

DISPERSION_SECONDS_MHZ = 4148.808


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def delays(frequencies, tsamp: float, dm: float) -> np.ndarray:
    f = _d(frequencies)
    out = np.empty(f.size, dtype=np.uint64)
    check(lib().psr_delays(f.ctypes.data_as(C.POINTER(C.c_double)), C.c_uint64(f.size),
                           C.c_double(tsamp), C.c_double(dm),
                           out.ctypes.data_as(C.POINTER(C.c_uint64))))
    return out


def dm_step(frequencies, tsamp: float) -> float:
    f = _d(frequencies)
    out = C.c_double()
    check(lib().psr_dm_step(f.ctypes.data_as(C.POINTER(C.c_double)), C.c_uint64(f.size),
                            C.c_double(tsamp), C.byref(out)))
    return out.value


def plan(dm_min: float, dm_max: float, step: float) -> np.ndarray:
    n = C.c_uint64()
    check(lib().psr_plan(C.c_double(dm_min), C.c_double(dm_max), C.c_double(step), None,
                         C.c_uint64(0), C.byref(n)))
    out = np.empty(n.value, dtype=np.float64)
    check(lib().psr_plan(C.c_double(dm_min), C.c_double(dm_max), C.c_double(step),
                         out.ctypes.data_as(C.POINTER(C.c_double)), C.c_uint64(out.size),
                         C.byref(n)))
    return out


def apply(fb: Filterbank, d, length: int | None = None) -> np.ndarray:
    dd = np.ascontiguousarray(d, dtype=np.uint64)
    n = C.c_uint64()
    lng = C.c_int64(-1 if length is None else int(length))
    check(lib().psr_dedisperse(fb.handle, dd.ctypes.data_as(C.POINTER(C.c_uint64)), lng, None,
                               C.c_uint64(0), C.byref(n)))
    out = np.empty(n.value, dtype=np.float32)
    check(lib().psr_dedisperse(fb.handle, dd.ctypes.data_as(C.POINTER(C.c_uint64)), lng,
                               out.ctypes.data_as(C.POINTER(C.c_float)), C.c_uint64(out.size),
                               C.byref(n)))
    return out


def apply_trials(fb: Filterbank, trials, length: int, with_sums: bool = False):
    """Series of every trial DM, [ntrials][length]; with_sums also returns
    each series' f64 sum (the one periodicity's mean uses)."""
    t = _d(trials)
    out = np.empty((t.size, int(length)), dtype=np.float32)
    sums = np.empty(t.size, dtype=np.float64)
    check(lib().psr_dedisperse_trials(fb.handle, t.ctypes.data_as(C.POINTER(C.c_double)),
                                      C.c_uint64(t.size), C.c_uint64(length),
                                      out.ctypes.data_as(C.POINTER(C.c_float)),
                                      sums.ctypes.data_as(C.POINTER(C.c_double))
                                      if with_sums else None))
    return (out, sums) if with_sums else out


def test_stage_timeout(fb: Filterbank, spin_limit: int = 1000) -> None:
    """Test hook (psr_test_stage_timeout): one dedispersion launch whose TMA
    barriers are armed but never fed, so the bounded waits run out; raises
    WaitTimeout as a real give-up would."""
    check(lib().psr_test_stage_timeout(fb.handle, C.c_uint64(spin_limit)))


def set_subbands(subbands: int) -> None:
    """Process-wide dedispersion tuning for samples stored in 8 bits
    (psr_set_dedisp_subbands): 0 = channel by channel, 4 or 8 = subband
    reuse, -1 = the library default.  Results are identical either way."""
    check(lib().psr_set_dedisp_subbands(C.c_int(subbands)))
