"""ORACLE - test infrastructure only.

ctypes view of oracle/_build/liboracle.so, the CPU restatement of the
PulsarSr search path (see psr_oracle.h for what is pinned and how).  Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module, and only as the checker.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")


class Header(C.Structure):
    _fields_ = [("nchans", C.c_int64), ("nbits", C.c_int64), ("tsamp", C.c_double),
                ("fch1", C.c_double), ("foff", C.c_double), ("data_offset", C.c_int64)]


class Candidate(C.Structure):
    _fields_ = [("frequency_hz", C.c_double), ("period_s", C.c_double), ("dm", C.c_double),
                ("harmonics", C.c_uint64), ("score", C.c_double)]


class Config(C.Structure):
    _fields_ = [("min_hz", C.c_double), ("max_hz", C.c_double), ("threshold", C.c_double),
                ("max_candidates", C.c_uint64), ("birdies", C.POINTER(C.c_double)),
                ("nbirdies", C.c_uint64), ("max_harmonics", C.c_uint64)]


class ProfileStats(C.Structure):
    _fields_ = [("period_s", C.c_double), ("snr", C.c_double),
                ("reduced_chi_square", C.c_double)]


class Measurement(C.Structure):
    _fields_ = [("snr", C.c_double), ("on_samples", C.c_uint64), ("off_samples", C.c_uint64),
                ("mean_difference", C.c_double), ("standard_error", C.c_double)]


CAND_DTYPE = np.dtype([("frequency_hz", "<f8"), ("period_s", "<f8"), ("dm", "<f8"),
                       ("harmonics", "<u8"), ("score", "<f8")])

_lib = None


def build() -> str:
    """Compile the oracle with its Makefile (g++ only)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _lib.orc_last_error.restype = C.c_char_p
        _lib.orc_median.restype = C.c_float
        _lib.orc_psr_search_json.restype = C.c_void_p
        _lib.orc_analyze_json.restype = C.c_void_p
    return _lib


class OracleError(RuntimeError):
    pass


def _check(rc: int) -> None:
    if rc != 0:
        raise OracleError(lib().orc_last_error().decode())


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(C.POINTER(t))


def parse_header(data: bytes) -> dict:
    h = Header()
    _check(lib().orc_parse_header(data, C.c_uint64(len(data)), C.byref(h)))
    return {k: getattr(h, k) for k, _ in Header._fields_}


def decode(data: bytes, limit: int | None = None):
    """fbank::decode -> (header dict, channel-major float32 array [nchans, nsamples])."""
    h = Header()
    ns = C.c_uint64()
    lim = C.c_int64(-1 if limit is None else int(limit))
    _check(lib().orc_decode(data, C.c_uint64(len(data)), lim, C.byref(h), C.byref(ns), None))
    out = np.empty(h.nchans * ns.value, dtype=np.float32)
    _check(lib().orc_decode(data, C.c_uint64(len(data)), lim, C.byref(h), C.byref(ns),
                            _ptr(out, C.c_float)))
    hd = {k: getattr(h, k) for k, _ in Header._fields_}
    return hd, out.reshape(h.nchans, ns.value)


def median(values) -> float:
    v = _f32(values)
    return float(lib().orc_median(_ptr(v, C.c_float), C.c_uint64(v.size)))


def channel_stats(data: np.ndarray):
    """rfi::mask's channel means and variances (reference-order f32 sums)."""
    d = _f32(data)
    nch, ns = d.shape
    m = np.empty(nch, dtype=np.float32)
    v = np.empty(nch, dtype=np.float32)
    _check(lib().orc_channel_stats(_ptr(d, C.c_float), C.c_uint64(nch), C.c_uint64(ns),
                                   _ptr(m, C.c_float), _ptr(v, C.c_float)))
    return m, v


def rfi_mask(data: np.ndarray, block_samples: int, threshold: float):
    """rfi::mask on a copy; returns (masked data, dict)."""
    d = np.array(data, dtype=np.float32, order="C", copy=True)
    nch, ns = d.shape
    ch = np.empty(nch, dtype=np.uint64)
    nb = -(-ns // block_samples)
    bl = np.empty(nb, dtype=np.uint64)
    nc, nbb, frac = C.c_uint64(), C.c_uint64(), C.c_double()
    _check(lib().orc_rfi_mask(_ptr(d, C.c_float), C.c_uint64(nch), C.c_uint64(ns),
                              C.c_uint64(block_samples), C.c_float(threshold),
                              _ptr(ch, C.c_uint64), C.byref(nc), _ptr(bl, C.c_uint64),
                              C.c_uint64(nb), C.byref(nbb), C.byref(frac)))
    return d, {"channels": [int(x) for x in ch[:nc.value]],
               "blocks": [int(x) for x in bl[:nbb.value]],
               "block_samples": int(block_samples), "masked_fraction": frac.value}


def delays(freqs, tsamp: float, dm: float) -> np.ndarray:
    f = np.ascontiguousarray(freqs, dtype=np.float64)
    out = np.empty(f.size, dtype=np.uint64)
    _check(lib().orc_delays(_ptr(f, C.c_double), C.c_uint64(f.size), C.c_double(tsamp),
                            C.c_double(dm), _ptr(out, C.c_uint64)))
    return out


def dm_step(freqs, tsamp: float) -> float:
    f = np.ascontiguousarray(freqs, dtype=np.float64)
    out = C.c_double()
    _check(lib().orc_dm_step(_ptr(f, C.c_double), C.c_uint64(f.size), C.c_double(tsamp),
                             C.byref(out)))
    return out.value


def plan(dm_min: float, dm_max: float, step: float) -> np.ndarray:
    n = C.c_uint64()
    _check(lib().orc_plan(C.c_double(dm_min), C.c_double(dm_max), C.c_double(step), None,
                          C.c_uint64(0), C.byref(n)))
    out = np.empty(n.value, dtype=np.float64)
    _check(lib().orc_plan(C.c_double(dm_min), C.c_double(dm_max), C.c_double(step),
                          _ptr(out, C.c_double), C.c_uint64(out.size), C.byref(n)))
    return out


def apply(data: np.ndarray, d, length: int | None = None) -> np.ndarray:
    x = _f32(data)
    nch, ns = x.shape
    dd = np.ascontiguousarray(d, dtype=np.uint64)
    n = C.c_uint64()
    lng = C.c_int64(-1 if length is None else int(length))
    _check(lib().orc_apply(_ptr(x, C.c_float), C.c_uint64(nch), C.c_uint64(ns),
                           _ptr(dd, C.c_uint64), lng, None, C.byref(n)))
    out = np.empty(n.value, dtype=np.float32)
    _check(lib().orc_apply(_ptr(x, C.c_float), C.c_uint64(nch), C.c_uint64(ns),
                           _ptr(dd, C.c_uint64), lng, _ptr(out, C.c_float), C.byref(n)))
    return out


def fft_size(length: int) -> int:
    return 1 << (max(int(length) - 1, 0)).bit_length() << 1 if length > 1 else 2


def raw_power(series) -> np.ndarray:
    s = _f32(series)
    n = 2 * (1 << (s.size - 1).bit_length())
    out = np.empty(n // 2 + 1, dtype=np.float32)
    _check(lib().orc_raw_power(_ptr(s, C.c_float), C.c_uint64(s.size), _ptr(out, C.c_float)))
    return out


def raw_power_f64(series) -> np.ndarray:
    s = _f32(series)
    n = 2 * (1 << (s.size - 1).bit_length())
    out = np.empty(n // 2 + 1, dtype=np.float64)
    _check(lib().orc_raw_power_f64(_ptr(s, C.c_float), C.c_uint64(s.size),
                                   _ptr(out, C.c_double)))
    return out


def make_config(min_hz=1.0, max_hz=float("inf"), threshold=6.0, max_candidates=32,
                birdies=(), max_harmonics=16):
    b = np.ascontiguousarray(np.array(birdies, dtype=np.float64).reshape(-1))
    cfg = Config(min_hz, max_hz, threshold, max_candidates,
                 _ptr(b, C.c_double) if b.size else None, b.size // 2, max_harmonics)
    cfg._keep = b  # keep the birdie buffer alive with the struct
    return cfg


def periodicity(series, tsamp: float, dm: float, **cfg) -> np.ndarray:
    s = _f32(series)
    c = make_config(**cfg)
    n = C.c_uint64()
    cap = 4096
    out = np.empty(cap, dtype=CAND_DTYPE)
    _check(lib().orc_periodicity(_ptr(s, C.c_float), C.c_uint64(s.size), C.c_double(tsamp),
                                 C.c_double(dm), C.byref(c), out.ctypes.data_as(C.c_void_p),
                                 C.c_uint64(cap), C.byref(n)))
    return out[:n.value].copy()


def sift(cands: np.ndarray, resolution_hz: float, limit: int, reject_dm_zero: bool):
    c = np.ascontiguousarray(cands, dtype=CAND_DTYPE)
    out = np.empty(max(len(c), 1), dtype=CAND_DTYPE)
    n = C.c_uint64()
    _check(lib().orc_sift(c.ctypes.data_as(C.c_void_p), C.c_uint64(len(c)),
                          C.c_double(resolution_hz), C.c_uint64(limit),
                          C.c_int(1 if reject_dm_zero else 0),
                          out.ctypes.data_as(C.c_void_p), C.byref(n)))
    return out[:n.value].copy()


def profile_at(series, tsamp: float, period: float, bins: int, offset: int = 0):
    s = _f32(series)
    st = ProfileStats()
    vals = np.empty(bins, dtype=np.float32)
    cnt = np.empty(bins, dtype=np.uint64)
    _check(lib().orc_profile_at(_ptr(s, C.c_float), C.c_uint64(s.size), C.c_double(tsamp),
                                C.c_double(period), C.c_uint64(bins), C.c_uint64(offset),
                                C.byref(st), _ptr(vals, C.c_float), _ptr(cnt, C.c_uint64)))
    return {"period_s": st.period_s, "snr": st.snr,
            "reduced_chi_square": st.reduced_chi_square, "bins": vals, "counts": cnt}


def refine(series, tsamp: float, frequency: float, span_hz: float, steps: int, bins: int):
    s = _f32(series)
    st = ProfileStats()
    vals = np.empty(bins, dtype=np.float32)
    cnt = np.empty(bins, dtype=np.uint64)
    _check(lib().orc_refine(_ptr(s, C.c_float), C.c_uint64(s.size), C.c_double(tsamp),
                            C.c_double(frequency), C.c_double(span_hz), C.c_uint64(steps),
                            C.c_uint64(bins), C.byref(st), _ptr(vals, C.c_float),
                            _ptr(cnt, C.c_uint64)))
    return {"period_s": st.period_s, "snr": st.snr,
            "reduced_chi_square": st.reduced_chi_square, "bins": vals, "counts": cnt}


def measure(x, offset: int, tsamp: float, period: float, start_bin: int, width_bins: int,
            bins: int) -> dict:
    s = _f32(x)
    m = Measurement()
    _check(lib().orc_measure(_ptr(s, C.c_float), C.c_uint64(s.size), C.c_uint64(offset),
                             C.c_double(tsamp), C.c_double(period), C.c_uint64(start_bin),
                             C.c_uint64(width_bins), C.c_uint64(bins), C.byref(m)))
    return {k: getattr(m, k) for k, _ in Measurement._fields_}


def search_trials(data: np.ndarray, freqs, tsamp: float, trials, discovery: int,
                  threads: int = 1, **cfg):
    """Per-trial candidate lists of the psr search loop, concatenated in order."""
    x = _f32(data)
    nch, ns = x.shape
    f = np.ascontiguousarray(freqs, dtype=np.float64)
    t = np.ascontiguousarray(trials, dtype=np.float64)
    c = make_config(**cfg)
    counts = np.zeros(t.size, dtype=np.uint64)
    cap = 32 * t.size + 1024
    out = np.empty(cap, dtype=CAND_DTYPE)
    ntot = C.c_uint64()
    _check(lib().orc_search_trials(_ptr(x, C.c_float), C.c_uint64(nch), C.c_uint64(ns),
                                   _ptr(f, C.c_double), C.c_double(tsamp), _ptr(t, C.c_double),
                                   C.c_uint64(t.size), C.c_uint64(discovery), C.byref(c),
                                   C.c_int(threads), _ptr(counts, C.c_uint64),
                                   out.ctypes.data_as(C.c_void_p), C.c_uint64(cap),
                                   C.byref(ntot)))
    return counts, out[:min(ntot.value, cap)].copy()


def psr_search(data: bytes, dm_min=0.0, dm_max=500.0, dm_step=None, min_hz=15.0,
               max_hz=2000.0, threshold=8.0, top=5, bins=64, no_rfi=False, birdies=(),
               max_samples=None, threads=1) -> dict:
    """`psr search` minus plots/hashing/files; returns the parsed JSON document."""
    b = np.ascontiguousarray(np.array(birdies, dtype=np.float64).reshape(-1))
    ptr = lib().orc_psr_search_json(
        data, C.c_uint64(len(data)), C.c_double(dm_min), C.c_double(dm_max),
        C.c_double(-1.0 if dm_step is None else dm_step), C.c_double(min_hz),
        C.c_double(max_hz), C.c_double(threshold), C.c_uint64(top), C.c_uint64(bins),
        C.c_int(1 if no_rfi else 0), _ptr(b, C.c_double) if b.size else None,
        C.c_uint64(b.size // 2), C.c_int64(-1 if max_samples is None else max_samples),
        C.c_int(threads))
    if not ptr:
        raise OracleError(lib().orc_last_error().decode())
    try:
        text = C.string_at(ptr).decode()
    finally:
        lib().orc_free(C.c_void_p(ptr))
    return json.loads(text)


def analyze(data: np.ndarray, freqs, tsamp: float, trials, generated, limit: int = 5,
            bins: int = 64) -> dict:
    """confirmation::analyze on masked channel-major data; the parsed Outcome."""
    x = _f32(data)
    nch, ns = x.shape
    f = np.ascontiguousarray(freqs, dtype=np.float64)
    t = np.ascontiguousarray(trials, dtype=np.float64)
    g = np.ascontiguousarray(np.asarray(generated, dtype=CAND_DTYPE))
    ptr = lib().orc_analyze_json(_ptr(x, C.c_float), C.c_uint64(nch), C.c_uint64(ns),
                                 _ptr(f, C.c_double), C.c_double(tsamp), _ptr(t, C.c_double),
                                 C.c_uint64(t.size), g.ctypes.data_as(C.c_void_p),
                                 C.c_uint64(g.size), C.c_uint64(limit), C.c_uint64(bins))
    if not ptr:
        raise OracleError(lib().orc_last_error().decode())
    try:
        text = C.string_at(ptr).decode()
    finally:
        lib().orc_free(C.c_void_p(ptr))
    return json.loads(text)


def refine_objective(data: np.ndarray, freqs, tsamp: float, n: int, period: float, pdot: float,
                     dm: float, bins: int = 128, subints: int = 64, variance: float = 0.0):
    """FP64 objective J and gradient (dJ/dP, dJ/dPdot, dJ/dDM) of the
    gradient-refinement model, and its profile."""
    x = _f32(data)
    nch, ns = x.shape
    f = np.ascontiguousarray(freqs, dtype=np.float64)
    J = C.c_double()
    grad = np.zeros(3)
    prof = np.zeros(bins)
    rc = lib().orc_refine_objective(_ptr(x, C.c_float), C.c_uint64(nch), C.c_uint64(ns),
                                    _ptr(f, C.c_double), C.c_double(tsamp), C.c_uint64(n),
                                    C.c_double(period), C.c_double(pdot), C.c_double(dm),
                                    C.c_uint64(bins), C.c_uint64(subints),
                                    C.c_double(variance), C.byref(J), _ptr(grad, C.c_double),
                                    _ptr(prof, C.c_double))
    _check(rc)
    return J.value, grad, prof
