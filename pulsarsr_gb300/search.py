"""search: GPU periodicity search, the batched trial loop and sifting.

Mirrors search::{Config, Candidate, periodicity, sift} (search/src/lib.rs:
6-176) and the psr search trial loop (cli/src/main.rs:462-473).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from ._lib import Candidate as _Cand
from ._lib import SearchConfig, check, lib
from .fbank import Filterbank

CAND_DTYPE = np.dtype([("frequency_hz", "<f8"), ("period_s", "<f8"), ("dm", "<f8"),
                       ("harmonics", "<u8"), ("score", "<f8")])


@dataclass
class Config:
    """search::Config (search/src/lib.rs:14-32) with the same defaults."""
    min_hz: float = 1.0
    max_hz: float = float("inf")
    threshold: float = 6.0
    max_candidates: int = 32
    birdies: list = field(default_factory=list)
    # Largest harmonic sum: 16 as the reference (h = 1, 2, 4, 8, 16); 32 adds
    # h = 32, an extension with the same score formula.
    max_harmonics: int = 16

    def _c(self) -> SearchConfig:
        b = np.ascontiguousarray(np.array(self.birdies, dtype=np.float64).reshape(-1))
        cfg = SearchConfig(self.min_hz, self.max_hz, self.threshold, self.max_candidates,
                           b.ctypes.data_as(C.POINTER(C.c_double)) if b.size else None,
                           b.size // 2, self.max_harmonics)
        cfg._keep = b
        return cfg


def raw_power(series) -> np.ndarray:
    """Raw |X|^2 of the zero-padded, mean-removed series (search/src/lib.rs:35-44)."""
    s = np.ascontiguousarray(series, dtype=np.float32)
    n = 2 * (1 << (s.size - 1).bit_length())
    out = np.empty(n // 2 + 1, dtype=np.float32)
    check(lib().psr_raw_power(s.ctypes.data_as(C.POINTER(C.c_float)), C.c_uint64(s.size),
                              out.ctypes.data_as(C.POINTER(C.c_float))))
    return out


def periodicity(series, tsamp: float, dm: float, config: Config | None = None) -> np.ndarray:
    config = config or Config()
    s = np.ascontiguousarray(series, dtype=np.float32)
    cfg = config._c()
    cap = max(int(config.max_candidates), 1)
    out = np.empty(cap, dtype=CAND_DTYPE)
    n = C.c_uint64()
    check(lib().psr_periodicity(s.ctypes.data_as(C.POINTER(C.c_float)), C.c_uint64(s.size),
                                C.c_double(tsamp), C.c_double(dm), C.byref(cfg),
                                out.ctypes.data_as(C.c_void_p), C.c_uint64(cap), C.byref(n)))
    return out[:n.value].copy()


def search_trials(fb: Filterbank, trials, discovery: int, config: Config):
    """(counts per trial, candidates in trial order) for every trial DM."""
    t = np.ascontiguousarray(trials, dtype=np.float64)
    cfg = config._c()
    counts = np.zeros(t.size, dtype=np.uint64)
    cap = t.size * max(int(config.max_candidates), 1)
    out = np.empty(max(cap, 1), dtype=CAND_DTYPE)
    n = C.c_uint64()
    check(lib().psr_search_trials(fb.handle, t.ctypes.data_as(C.POINTER(C.c_double)),
                                  C.c_uint64(t.size), C.c_uint64(discovery), C.byref(cfg),
                                  counts.ctypes.data_as(C.POINTER(C.c_uint64)),
                                  out.ctypes.data_as(C.c_void_p), C.c_uint64(cap), C.byref(n)))
    return counts, out[:n.value].copy()


def sift(candidates, resolution_hz: float, limit: int, reject_dm_zero: bool) -> np.ndarray:
    c = np.ascontiguousarray(candidates, dtype=CAND_DTYPE)
    out = np.empty(max(len(c), 1), dtype=CAND_DTYPE)
    n = C.c_uint64()
    check(lib().psr_sift(c.ctypes.data_as(C.c_void_p), C.c_uint64(len(c)),
                         C.c_double(resolution_hz), C.c_uint64(limit),
                         C.c_int(1 if reject_dm_zero else 0), out.ctypes.data_as(C.c_void_p),
                         C.byref(n)))
    return out[:n.value].copy()
