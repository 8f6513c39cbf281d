"""fbank: SIGPROC header parsing and device-resident decoding.

Mirrors fbank::{parse_header, decode, read, read_header}
(fbank/src/lib.rs:72-209).  decode() parses the header on the host, copies
the packed payload to the GPU once and unpacks it there; the samples stay in
HBM, channel-major, for the rest of the pipeline.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import Header, check, lib


@dataclass
class HeaderInfo:
    nchans: int
    nbits: int
    tsamp: float
    fch1: float
    foff: float
    data_offset: int

    def frequencies(self) -> np.ndarray:
        """fbank::Header::frequencies (fbank/src/lib.rs:40-44)."""
        return self.fch1 + np.arange(self.nchans, dtype=np.float64) * self.foff


def _hdr(h: Header) -> HeaderInfo:
    return HeaderInfo(h.nchans, h.nbits, h.tsamp, h.fch1, h.foff, h.data_offset)


def parse_header(data: bytes) -> HeaderInfo:
    h = Header()
    check(lib().psr_parse_header(data, C.c_uint64(len(data)), C.byref(h)))
    return _hdr(h)


class Filterbank:
    """A decoded filterbank whose samples live on the GPU (fbank::Filterbank)."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)
        h = Header()
        ns = C.c_uint64()
        check(lib().psr_fb_info(self._h, C.byref(h), C.byref(ns)))
        self.header = _hdr(h)
        self.nsamples = int(ns.value)

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    @property
    def data(self) -> np.ndarray:
        """Channel-major f32 samples, shape (nchans, nsamples) (a host copy)."""
        out = np.empty(self.header.nchans * self.nsamples, dtype=np.float32)
        check(lib().psr_fb_download(self._h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out.reshape(self.header.nchans, self.nsamples)

    def channels(self, c0: int, count: int) -> np.ndarray:
        """Channels [c0, c0 + count) as f32, shape (count, nsamples) (a host copy)."""
        out = np.empty((int(count), self.nsamples), dtype=np.float32)
        check(lib().psr_fb_download_channels(self._h, C.c_uint64(c0), C.c_uint64(count),
                                             out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def channel(self, c: int) -> np.ndarray:
        return self.channels(c, 1)[0]

    def close(self) -> None:
        if self._h:
            lib().psr_fb_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def decode(data: bytes, limit: int | None = None) -> Filterbank:
    out = C.c_void_p()
    check(lib().psr_fb_decode(data, C.c_uint64(len(data)),
                              C.c_int64(-1 if limit is None else int(limit)), C.byref(out)))
    return Filterbank(out.value)


def read(path: str, limit: int | None = None) -> Filterbank:
    """fbank::read (fbank/src/lib.rs:198-203): the payload streams from the
    file to the device in chunks (psr_fb_read) and is unpacked there."""
    import os
    h = C.c_void_p()
    check(lib().psr_fb_read(os.fsencode(path), C.c_int64(-1 if limit is None else limit),
                            C.byref(h)))
    return Filterbank(h.value)


def read_header(path: str) -> HeaderInfo:
    with open(path, "rb") as f:
        return parse_header(f.read(65536))
