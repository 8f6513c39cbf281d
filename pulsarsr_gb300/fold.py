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


# ------------------------------------------------ gradient refinement
class Timing(C.Structure):
    """(P, Pdot, DM) of a refinement (psr_timing)."""
    _fields_ = [("period_s", C.c_double), ("pdot", C.c_double), ("dm", C.c_double)]


class RefineOptions(C.Structure):
    _fields_ = [("bins", C.c_uint64), ("subints", C.c_uint64), ("max_evals", C.c_uint64),
                ("tol_bins", C.c_double), ("exact", C.c_int32), ("dm_window", C.c_double)]

    @staticmethod
    def make(bins=128, subints=64, max_evals=40, tol_bins=1e-3, exact=False,
             dm_window=0.0) -> "RefineOptions":
        return RefineOptions(bins, subints, max_evals, tol_bins, 1 if exact else 0, dm_window)


TIMING_DTYPE = np.dtype([("period_s", "<f8"), ("pdot", "<f8"), ("dm", "<f8")])


def refine_objective(fb, n: int, period: float, pdot: float, dm: float, bins: int = 128,
                     subints: int = 64, variance: float = 0.0):
    """The gradient-refinement objective J, dJ/d(P, Pdot, DM), the profile and
    the (subints x bins) folded cells, computed on the device."""
    th = Timing(period, pdot, dm)
    opt = RefineOptions.make(bins, subints)
    J = C.c_double()
    grad = np.zeros(3)
    prof = np.zeros(bins)
    cells = np.zeros(bins * subints)
    check(lib().psr_refine_objective(fb.handle, C.c_uint64(n), C.byref(th), C.byref(opt),
                                     C.c_double(variance), C.byref(J),
                                     grad.ctypes.data_as(C.POINTER(C.c_double)),
                                     prof.ctypes.data_as(C.POINTER(C.c_double)),
                                     cells.ctypes.data_as(C.POINTER(C.c_double))))
    return J.value, grad, prof, cells.reshape(subints, bins)


def refine_cube_objective(fb, n: int, reference, points, bins: int = 128, subints: int = 64):
    """The cube objective of refine_gradient's default path: the cube folded
    at `reference` (P, Pdot, DM), J and dJ/d(P, Pdot, DM) at each point;
    returns (J array, gradient array of shape (npoints, 3))."""
    ref = Timing(*reference)
    pts = np.ascontiguousarray(np.array([tuple(x) for x in points], dtype=TIMING_DTYPE))
    J = np.zeros(pts.size)
    grad = np.zeros((pts.size, 3))
    opt = RefineOptions.make(bins, subints)
    check(lib().psr_refine_cube_objective(fb.handle, C.c_uint64(n), C.byref(ref),
                                          pts.ctypes.data_as(C.c_void_p), C.c_uint64(pts.size),
                                          C.byref(opt), J.ctypes.data_as(C.POINTER(C.c_double)),
                                          grad.ctypes.data_as(C.POINTER(C.c_double))))
    return J, grad


def refine_gradient(fb, n: int, starts, bins: int = 128, subints: int = 64,
                    max_evals: int = 40, tol_bins: float = 1e-3, exact: bool = False,
                    dm_window: float = 0.0):
    """Gradient refinement of every starting point (a TIMING_DTYPE array or
    (P, Pdot, DM) tuples); returns (refined, J, evaluations).  exact=False
    optimises on a folded cube per group of nearby starts, exact=True on the
    filterbank objective at every evaluation."""
    s = np.ascontiguousarray(np.array([tuple(x) for x in starts], dtype=TIMING_DTYPE))
    out = np.zeros_like(s)
    J = np.zeros(s.size)
    ev = np.zeros(s.size, dtype=np.uint64)
    opt = RefineOptions.make(bins, subints, max_evals, tol_bins, exact, dm_window)
    check(lib().psr_refine_gradient(fb.handle, C.c_uint64(n), s.ctypes.data_as(C.c_void_p),
                                    C.c_uint64(s.size), C.byref(opt),
                                    out.ctypes.data_as(C.c_void_p),
                                    J.ctypes.data_as(C.POINTER(C.c_double)),
                                    ev.ctypes.data_as(C.POINTER(C.c_uint64))))
    return out, J, ev


def refine_grid(fb, n: int, starts, resolution_hz: float, dm_step: float, dm_lo: float,
                dm_hi: float, bins: int = 64):
    """The reference's grid refinement (41 frequencies, then 21 half-step DMs)
    of every starting point, on the device; returns (refined, reduced chi2)."""
    s = np.ascontiguousarray(np.array([tuple(x) for x in starts], dtype=TIMING_DTYPE))
    out = np.zeros_like(s)
    r = np.zeros(s.size)
    check(lib().psr_refine_grid(fb.handle, C.c_uint64(n), s.ctypes.data_as(C.c_void_p),
                                C.c_uint64(s.size), C.c_double(resolution_hz),
                                C.c_double(dm_step), C.c_double(dm_lo), C.c_double(dm_hi),
                                C.c_uint64(bins), out.ctypes.data_as(C.c_void_p),
                                r.ctypes.data_as(C.POINTER(C.c_double))))
    return out, r
