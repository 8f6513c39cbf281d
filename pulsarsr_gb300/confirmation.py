"""search::confirmation mirror: group, analyze and the Outcome
(search/src/confirmation.rs:1-538), computed by libpsr on the device.

analyze() returns an Outcome whose .json() is the reference's serde_json
text (same field order and number format) and whose .data is that JSON
parsed into Python objects.
"""
from __future__ import annotations

import ctypes as C
import json
from dataclasses import dataclass

import numpy as np

from ._lib import check, lib
from .search import CAND_DTYPE


class Rules(C.Structure):
    """confirmation::Rules (confirmation.rs:17-40); version split-confirm-v1."""
    _fields_ = [("minimum_validation_snr", C.c_double), ("minimum_part_snr", C.c_double),
                ("minimum_time_parts", C.c_uint64), ("minimum_subbands", C.c_uint64),
                ("minimum_dm_contrast", C.c_double), ("minimum_dispersion_widths", C.c_double),
                ("maximum_zero_dm_spectral_ratio", C.c_double)]

    @staticmethod
    def default() -> "Rules":
        r = Rules()
        lib().psr_rules_default(C.byref(r))
        return r


class _Info(C.Structure):
    _fields_ = [("discovery_samples", C.c_uint64), ("validation_start_sample", C.c_uint64),
                ("validation_samples", C.c_uint64), ("common_samples", C.c_uint64),
                ("trial_count", C.c_uint64), ("candidates", C.c_uint64)]


def _cands(generated) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(generated, dtype=CAND_DTYPE))


@dataclass
class Family:
    leader: np.void
    members: np.ndarray


def group(candidates, resolution: float, limit: int) -> list[Family]:
    """confirmation::group (confirmation.rs:177-199)."""
    c = _cands(candidates)
    order = np.zeros(max(c.size, 1), dtype=np.uint64)
    fam = np.zeros(max(c.size, 1), dtype=np.int64)
    nf = C.c_uint64()
    check(lib().psr_group(c.ctypes.data_as(C.c_void_p), C.c_uint64(c.size),
                          C.c_double(resolution), C.c_uint64(limit),
                          order.ctypes.data_as(C.POINTER(C.c_uint64)),
                          fam.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(nf)))
    out = []
    sorted_c = c[order[:c.size].astype(np.int64)]
    for f in range(nf.value):
        members = sorted_c[fam[:c.size] == f]
        out.append(Family(members[0], members))
    return out


class Outcome:
    """confirmation::Outcome owned by libpsr."""

    def __init__(self, handle: C.c_void_p):
        self._o = handle
        info = _Info()
        check(lib().psr_outcome_info_get(self._o, C.byref(info)))
        self.discovery_samples = info.discovery_samples
        self.validation_start_sample = info.validation_start_sample
        self.validation_samples = info.validation_samples
        self.common_samples = info.common_samples
        self.trial_count = info.trial_count
        self.ncandidates = info.candidates
        self._data = None

    def json(self, pretty: bool = False) -> str:
        L = lib()
        n = L.psr_outcome_json(self._o, C.c_int(int(pretty)), None, C.c_uint64(0))
        buf = C.create_string_buffer(n + 1)
        L.psr_outcome_json(self._o, C.c_int(int(pretty)), buf, C.c_uint64(n + 1))
        return buf.value.decode()

    @property
    def data(self) -> dict:
        if self._data is None:
            self._data = json.loads(self.json())
        return self._data

    def close(self) -> None:
        if self._o:
            lib().psr_outcome_free(self._o)
            self._o = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _setup():
    L = lib()
    L.psr_outcome_json.restype = C.c_uint64
    L.psr_outcome_json.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_uint64]
    L.psr_outcome_free.argtypes = [C.c_void_p]
    L.psr_outcome_info_get.argtypes = [C.c_void_p, C.c_void_p]
    L.psr_rules_default.argtypes = [C.c_void_p]
    return L


def analyze(fb, trials, generated, limit: int = 5, bins: int = 64,
            rules: Rules | None = None) -> Outcome:
    """confirmation::analyze (confirmation.rs:203-496) on a device filterbank."""
    L = _setup()
    t = np.ascontiguousarray(trials, dtype=np.float64)
    c = _cands(generated)
    h = C.c_void_p()
    check(L.psr_analyze(fb.handle, t.ctypes.data_as(C.POINTER(C.c_double)), C.c_uint64(t.size),
                        c.ctypes.data_as(C.c_void_p), C.c_uint64(c.size), C.c_uint64(limit),
                        C.c_uint64(bins), C.byref(rules) if rules is not None else None,
                        C.byref(h)))
    return Outcome(h)


def analyze_session(sess, limit: int = 5, bins: int = 64, rules: Rules | None = None) -> Outcome:
    """analyze over a session's last run (the psr search command)."""
    L = _setup()
    h = C.c_void_p()
    check(L.psr_session_analyze(sess._s, C.c_uint64(limit), C.c_uint64(bins),
                                C.byref(rules) if rules is not None else None, C.byref(h)))
    return Outcome(h)
