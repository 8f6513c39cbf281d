"""fold: GPU phase folding, grid refinement and fixed-window measurement.

Mirrors fold::{profile, profile_at, refine} (fold/src/lib.rs:12-97) and
search::confirmation::measure (search/src/confirmation.rs:107-141).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import Measurement, ProfileStats, check, lib


def _prof(st: ProfileStats, vals, cnt) -> dict:
    return {"period_s": st.period_s, "snr": st.snr,
            "reduced_chi_square": st.reduced_chi_square, "bins": vals, "counts": cnt}


def profile_at(series, tsamp: float, period: float, bins: int, sample_offset: int = 0) -> dict:
    s = np.ascontiguousarray(series, dtype=np.float32)
    st = ProfileStats()
    vals = np.empty(bins, dtype=np.float32)
    cnt = np.empty(bins, dtype=np.uint64)
    check(lib().psr_profile_at(s.ctypes.data_as(C.POINTER(C.c_float)), C.c_uint64(s.size),
                               C.c_double(tsamp), C.c_double(period), C.c_uint64(bins),
                               C.c_uint64(sample_offset), C.byref(st),
                               vals.ctypes.data_as(C.POINTER(C.c_float)),
                               cnt.ctypes.data_as(C.POINTER(C.c_uint64))))
    return _prof(st, vals, cnt)


def profile(series, tsamp: float, period: float, bins: int) -> dict:
    return profile_at(series, tsamp, period, bins, 0)


def refine(series, tsamp: float, frequency: float, span_hz: float, steps: int,
           bins: int) -> dict:
    s = np.ascontiguousarray(series, dtype=np.float32)
    st = ProfileStats()
    vals = np.empty(bins, dtype=np.float32)
    cnt = np.empty(bins, dtype=np.uint64)
    check(lib().psr_refine(s.ctypes.data_as(C.POINTER(C.c_float)), C.c_uint64(s.size),
                           C.c_double(tsamp), C.c_double(frequency), C.c_double(span_hz),
                           C.c_uint64(steps), C.c_uint64(bins), C.byref(st),
                           vals.ctypes.data_as(C.POINTER(C.c_float)),
                           cnt.ctypes.data_as(C.POINTER(C.c_uint64))))
    return _prof(st, vals, cnt)


def measure(x, offset: int, tsamp: float, period: float, start_bin: int, width_bins: int,
            bins: int) -> dict:
    s = np.ascontiguousarray(x, dtype=np.float32)
    m = Measurement()
    check(lib().psr_measure(s.ctypes.data_as(C.POINTER(C.c_float)), C.c_uint64(s.size),
                            C.c_uint64(offset), C.c_double(tsamp), C.c_double(period),
                            C.c_uint64(start_bin), C.c_uint64(width_bins), C.c_uint64(bins),
                            C.byref(m)))
    return {k: getattr(m, k) for k, _ in Measurement._fields_}
