"""A device-resident search session (psr_session_* in include/psr.h).

Holds one observation shape on the GPU with every buffer allocated once:
load() copies a packed payload, run() enqueues unpack -> RFI mask -> trial
loop, sync() waits, candidates()/mask() read the results.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import Header, check, lib
from .fbank import HeaderInfo
from .search import CAND_DTYPE, Config


class SearchSession:
    def __init__(self, header: HeaderInfo, nsamples: int, trials, discovery: int,
                 config: Config, rfi_block_samples: int = 0, rfi_threshold: float = 8.0):
        h = Header(header.nchans, header.nbits, header.tsamp, header.fch1, header.foff,
                   header.data_offset)
        self.trials = np.ascontiguousarray(trials, dtype=np.float64)
        self.config = config
        self.nchans = header.nchans
        self.nsamples = int(nsamples)
        self._cfg = config._c()
        out = C.c_void_p()
        check(lib().psr_session_create(C.byref(h), C.c_uint64(nsamples),
                                       self.trials.ctypes.data_as(C.POINTER(C.c_double)),
                                       C.c_uint64(self.trials.size), C.c_uint64(discovery),
                                       C.byref(self._cfg), C.c_uint64(rfi_block_samples),
                                       C.c_float(rfi_threshold), C.byref(out)))
        self._s = out

    def load(self, payload) -> None:
        buf = np.frombuffer(payload, dtype=np.uint8) if isinstance(payload, (bytes, bytearray,
                                                                             memoryview)) \
            else np.ascontiguousarray(payload, dtype=np.uint8)
        check(lib().psr_session_load(self._s, buf.ctypes.data_as(C.POINTER(C.c_uint8)),
                                     C.c_uint64(buf.size)))

    def run(self) -> None:
        check(lib().psr_session_run(self._s))

    def sync(self) -> None:
        check(lib().psr_session_sync(self._s))

    @property
    def stream(self) -> int:
        return int(lib().psr_session_stream(self._s) or 0)

    @property
    def payload_device_ptr(self) -> int:
        return int(lib().psr_session_payload_device(self._s) or 0)

    def candidates(self):
        cap = self.trials.size * max(int(self.config.max_candidates), 1)
        counts = np.zeros(self.trials.size, dtype=np.uint64)
        out = np.empty(max(cap, 1), dtype=CAND_DTYPE)
        n = C.c_uint64()
        check(lib().psr_session_candidates(self._s, counts.ctypes.data_as(C.POINTER(C.c_uint64)),
                                           out.ctypes.data_as(C.c_void_p), C.c_uint64(cap),
                                           C.byref(n)))
        return counts, out[:n.value]

    def mask(self) -> dict:
        ch = np.zeros(self.nchans, dtype=np.uint64)
        bl = np.zeros(self.nsamples // 32 + 2, dtype=np.uint64)
        nc, nb, frac = C.c_uint64(), C.c_uint64(), C.c_double()
        check(lib().psr_session_mask(self._s, ch.ctypes.data_as(C.POINTER(C.c_uint64)),
                                     C.byref(nc), bl.ctypes.data_as(C.POINTER(C.c_uint64)),
                                     C.c_uint64(bl.size), C.byref(nb), C.byref(frac)))
        return {"channels": [int(x) for x in ch[:nc.value]],
                "blocks": [int(x) for x in bl[:nb.value]], "masked_fraction": frac.value}

    STAGES = ("unpack", "rfi", "dedisperse", "fft", "spectrum")

    def set_profiling(self, enable) -> None:
        """False/0: off; True/1: stage events, stages overlapping as usual;
        2: stage events with the stages serialised (each stage's own time)."""
        check(lib().psr_session_set_profiling(self._s, C.c_int(int(enable))))

    def stage_times(self, reset: bool = False) -> dict:
        ms = np.zeros(5, dtype=np.float64)
        n = np.zeros(5, dtype=np.uint64)
        check(lib().psr_session_stage_times(self._s, ms.ctypes.data_as(C.POINTER(C.c_double)),
                                            n.ctypes.data_as(C.POINTER(C.c_uint64)),
                                            C.c_int(1 if reset else 0)))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(self.STAGES)}

    def close(self) -> None:
        if self._s:
            lib().psr_session_free(self._s)
            self._s = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
