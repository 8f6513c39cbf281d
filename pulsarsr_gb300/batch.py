"""Batched search of many observations of uneven shape through one CUDA
graph launch (psr_batch_*).  Each observation is searched exactly as
search.search_trials / the session would search it."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import Header, SearchConfig, check, lib
from .search import CAND_DTYPE


class _Obs(C.Structure):
    _fields_ = [("header", Header), ("nsamples", C.c_uint64),
                ("trials", C.POINTER(C.c_double)), ("ntrials", C.c_uint64),
                ("discovery", C.c_uint64), ("config", SearchConfig),
                ("rfi_block_samples", C.c_uint64), ("rfi_threshold", C.c_float)]


class Batch:
    def __init__(self, observations, hbm_budget_bytes: int = 0):
        """observations: iterable of dicts with keys header (fbank.HeaderInfo),
        nsamples, trials, discovery, config (search.Config), rfi_block
        (0 = no masking) and rfi_threshold."""
        L = lib()
        L.psr_batch_stream.restype = C.c_void_p
        L.psr_batch_stream.argtypes = [C.c_void_p]
        L.psr_batch_free.argtypes = [C.c_void_p]
        self._keep = []
        arr = (_Obs * len(observations))()
        for i, o in enumerate(observations):
            h = o["header"]
            t = np.ascontiguousarray(o["trials"], dtype=np.float64)
            cfg = o["config"]._c()
            self._keep += [t, cfg]
            arr[i] = _Obs(Header(h.nchans, h.nbits, h.tsamp, h.fch1, h.foff, h.data_offset),
                          o["nsamples"], t.ctypes.data_as(C.POINTER(C.c_double)), t.size,
                          o["discovery"], cfg, o.get("rfi_block", 0),
                          o.get("rfi_threshold", 8.0))
        self.n = len(observations)
        self.ntrials = [len(o["trials"]) for o in observations]
        self._b = C.c_void_p()
        check(L.psr_batch_create(arr, C.c_uint64(self.n), C.c_uint64(hbm_budget_bytes),
                                 C.byref(self._b)))

    def load(self, i: int, payload) -> None:
        p = np.ascontiguousarray(np.frombuffer(payload, dtype=np.uint8)
                                 if isinstance(payload, (bytes, bytearray)) else payload,
                                 dtype=np.uint8)
        check(lib().psr_batch_load(self._b, C.c_uint64(i),
                                   p.ctypes.data_as(C.POINTER(C.c_uint8)), C.c_uint64(p.size)))

    def load_fb(self, i: int, fb) -> None:
        check(lib().psr_batch_load_fb(self._b, C.c_uint64(i), fb.handle))

    def tune(self):
        """psr_batch_tune: per shape class, the fastest (DM block, FFT launch
        size, subband width); returns the three per-observation arrays."""
        ch = np.zeros(self.n, dtype=np.uint64)
        inner = np.zeros(self.n, dtype=np.uint64)
        sub = np.zeros(self.n, dtype=np.int32)
        check(lib().psr_batch_tune(self._b, ch.ctypes.data_as(C.POINTER(C.c_uint64)),
                                   inner.ctypes.data_as(C.POINTER(C.c_uint64)),
                                   sub.ctypes.data_as(C.POINTER(C.c_int))))
        return ch, inner, sub

    def set_chunking(self, i: int, chunk: int, inner: int = 0) -> None:
        """Pin observation i's DM block and FFT launch size (trials)."""
        check(lib().psr_batch_set_chunking(self._b, C.c_uint64(i), C.c_uint64(chunk),
                                           C.c_uint64(inner)))

    def run(self) -> None:
        check(lib().psr_batch_run(self._b))

    def sync(self) -> None:
        check(lib().psr_batch_sync(self._b))

    @property
    def stream(self) -> int:
        return lib().psr_batch_stream(self._b)

    def candidates(self, i: int):
        counts = np.zeros(self.ntrials[i], dtype=np.uint64)
        cap = 64 * self.ntrials[i]
        out = np.empty(max(cap, 1), dtype=CAND_DTYPE)
        n = C.c_uint64()
        check(lib().psr_batch_candidates(self._b, C.c_uint64(i),
                                         counts.ctypes.data_as(C.POINTER(C.c_uint64)),
                                         out.ctypes.data_as(C.c_void_p), C.c_uint64(cap),
                                         C.byref(n)))
        return counts, out[:n.value].copy()

    def close(self) -> None:
        if self._b:
            lib().psr_batch_free(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
