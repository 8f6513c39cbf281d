"""Seeded synthetic SIGPROC filterbanks for the benchmark configurations.

The reference's own generator (synth/src/lib.rs:38-85) draws ChaCha8 noise
that cannot be regenerated here, and it only writes f32 files; the
configurations this build is measured on need quantised 8-bit and 4-bit
data with gains, interference and bursts, so this module is a new generator
(numpy PCG64, fixed seeds).  Pulses use the reference's physical (fractional)
dispersion delay K*DM*(f^-2 - f_ref^-2) and a Gaussian of the given duty
cycle (FWHM), as in synth/src/lib.rs:56-62.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

K_DM = 4148.808


def _s(text: str) -> bytes:
    b = text.encode()
    return struct.pack("<i", len(b)) + b


def header_bytes(nchans: int, nbits: int, tsamp: float, fch1: float, foff: float,
                 source_name: str = "seeded synthetic", tstart: float = 60000.0) -> bytes:
    """A SIGPROC header accepted by fbank::parse_header (fbank/src/lib.rs:72-147)."""
    out = _s("HEADER_START")
    out += _s("source_name") + _s(source_name)
    for k, v in (("machine_id", 0), ("telescope_id", 0), ("data_type", 1), ("nchans", nchans),
                 ("nbits", nbits), ("nifs", 1)):
        out += _s(k) + struct.pack("<i", v)
    for k, v in (("tstart", tstart), ("tsamp", tsamp), ("fch1", fch1), ("foff", foff)):
        out += _s(k) + struct.pack("<d", v)
    out += _s("HEADER_END")
    return out


def pack(values: np.ndarray, nbits: int) -> bytes:
    """Pack time-major samples (shape (nsamples, nchans)) SIGPROC-style:
    sub-byte samples least-significant bits first, 16-bit little endian."""
    v = np.ascontiguousarray(values).reshape(-1)
    if nbits == 32:
        return np.ascontiguousarray(v, dtype="<f4").tobytes()
    if nbits == 16:
        return np.ascontiguousarray(v, dtype="<u2").tobytes()
    if nbits == 8:
        return np.ascontiguousarray(v, dtype=np.uint8).tobytes()
    per = 8 // nbits
    u = np.ascontiguousarray(v, dtype=np.uint8)
    if u.size % per:
        raise ValueError("sample count does not fill whole bytes")
    u = u.reshape(-1, per)
    out = np.zeros(u.shape[0], dtype=np.uint8)
    for j in range(per):
        out |= (u[:, j] & ((1 << nbits) - 1)) << (j * nbits)
    return out.tobytes()


@dataclass
class Pulsar:
    period_s: float
    dm: float
    duty: float          # FWHM as a fraction of the period
    amplitude: float     # peak, in units of the noise sigma
    phase: float = 0.25
    pdot: float = 0.0    # period derivative (s/s); phase = t/P - pdot t^2 / (2 P^2)


@dataclass
class Observation:
    nchans: int
    nbits: int
    nsamples: int
    tsamp: float
    fch1: float
    foff: float
    seed: int
    noise_mean: float = 100.0
    noise_sigma: float = 10.0
    gain_spread: float = 0.0         # per-channel gain U(1-g, 1+g)
    pulsars: list = field(default_factory=list)
    tone_hz: float = 0.0             # zero-DM periodic interference
    tone_amplitude: float = 0.0      # in sigma
    bursts: int = 0                  # broadband zero-DM bursts
    burst_amplitude: float = 3.0     # in sigma
    burst_seconds: float = 0.05
    name: str = "seeded synthetic"

    def frequencies(self) -> np.ndarray:
        return self.fch1 + np.arange(self.nchans) * self.foff

    def samples(self) -> np.ndarray:
        """Quantised samples, time-major (nsamples, nchans)."""
        rng = np.random.Generator(np.random.PCG64(self.seed))
        nch, ns = self.nchans, self.nsamples
        gains = 1.0 + self.gain_spread * (2.0 * rng.random(nch) - 1.0)
        t = np.arange(ns, dtype=np.float64) * self.tsamp
        freqs = self.frequencies()
        ref = freqs.max()
        zero_dm = np.zeros(ns, dtype=np.float64)
        if self.tone_amplitude:
            zero_dm += self.tone_amplitude * np.sin(2 * np.pi * self.tone_hz * t)
        if self.bursts:
            width = max(int(self.burst_seconds / self.tsamp), 1)
            starts = rng.integers(0, max(ns - width, 1), self.bursts)
            for s in starts:
                zero_dm[s:s + width] += self.burst_amplitude
        hi = (1 << self.nbits) - 1 if self.nbits <= 16 else None
        out = np.empty((ns, nch), dtype=np.float32 if self.nbits == 32 else
                       (np.uint16 if self.nbits == 16 else np.uint8))
        for c in range(nch):
            x = rng.standard_normal(ns) + zero_dm
            for p in self.pulsars:
                delay = K_DM * p.dm * (freqs[c] ** -2 - ref ** -2)
                td = t - delay
                ph = np.mod(td / p.period_s - 0.5 * p.pdot * td * td / p.period_s ** 2
                            - p.phase, 1.0)
                dist = np.minimum(ph, 1.0 - ph)
                x += p.amplitude * np.exp(-0.5 * (dist / (p.duty / 2.355)) ** 2)
            v = self.noise_mean + self.noise_sigma * gains[c] * x
            if hi is None:
                out[:, c] = v.astype(np.float32)
            else:
                out[:, c] = np.clip(np.rint(v), 0, hi).astype(out.dtype)
        return out

    def header(self) -> bytes:
        return header_bytes(self.nchans, self.nbits, self.tsamp, self.fch1, self.foff, self.name)

    def to_bytes(self) -> bytes:
        return self.header() + pack(self.samples(), self.nbits)


def config_c1(seed: int = 1) -> Observation:
    """64 ch, 8-bit, 2^18 samples, 64 us, 1350-1450 MHz; N(100, 10); a 32 ms
    pulsar at DM 62 with 5% duty and 0.5 sigma amplitude."""
    return Observation(nchans=64, nbits=8, nsamples=1 << 18, tsamp=64e-6, fch1=1450.0,
                       foff=-1.5625, seed=seed, noise_mean=100.0, noise_sigma=10.0,
                       pulsars=[Pulsar(0.032, 62.0, 0.05, 0.5)], name="config1 synthetic")


def config_c2(seed: int = 2) -> Observation:
    """GBT L-band tutorial shape: 96 x 1 MHz channels, first channel at
    1447.5 MHz as in the tutorial file's header (so the default DM step gives
    the reference's 2000-trial plan over 0-500), 4-bit, 72 us, 531000
    samples; 4-bit noise around level 8 with +-20% channel gains; a 4.6214 ms
    pulsar at DM 62.4 (3% duty, folded SNR ~30), a 28.76 Hz zero-DM tone and
    5 broadband bursts."""
    return Observation(nchans=96, nbits=4, nsamples=531000, tsamp=72e-6, fch1=1447.5,
                       foff=-1.0, seed=seed, noise_mean=8.0, noise_sigma=2.0, gain_spread=0.2,
                       pulsars=[Pulsar(0.0046214, 62.4, 0.03, 0.04)], tone_hz=28.76,
                       tone_amplitude=0.05, bursts=5, burst_amplitude=1.0,
                       name="config2 GBT-shaped synthetic")


# ----------------------------------------------------------- on the device
def device(nchans: int, nbits: int, nsamples: int, tsamp: float, fch1: float, foff: float,
           seed: int, noise_mean: float = 0.0, noise_sigma: float = 1.0,
           gain_spread: float = 0.0, pulsars=()):
    """A seeded synthetic filterbank generated directly in HBM (psr_fb_synth);
    pulsars are Pulsar values.  Returns an fbank.Filterbank."""
    import ctypes as C

    from ._lib import check, lib
    from .fbank import Filterbank

    class _P(C.Structure):
        _fields_ = [("period_s", C.c_double), ("pdot", C.c_double), ("dm", C.c_double),
                    ("duty", C.c_double), ("amplitude", C.c_double), ("phase", C.c_double)]

    class _Cfg(C.Structure):
        _fields_ = [("nchans", C.c_int64), ("nbits", C.c_int64), ("nsamples", C.c_uint64),
                    ("tsamp", C.c_double), ("fch1", C.c_double), ("foff", C.c_double),
                    ("seed", C.c_uint64), ("noise_mean", C.c_double),
                    ("noise_sigma", C.c_double), ("gain_spread", C.c_double),
                    ("pulsars", C.POINTER(_P)), ("npulsars", C.c_uint64)]

    arr = (_P * max(len(pulsars), 1))(*[_P(p.period_s, p.pdot, p.dm, p.duty, p.amplitude,
                                            p.phase) for p in pulsars])
    cfg = _Cfg(nchans, nbits, nsamples, tsamp, fch1, foff, seed, noise_mean, noise_sigma,
               gain_spread, arr if pulsars else None, len(pulsars))
    h = C.c_void_p()
    check(lib().psr_fb_synth(C.byref(cfg), C.byref(h)))
    return Filterbank(h.value)


def inject_rfi(fb, seed: int, nb_channels: int = 0, nb_amplitude: float = 0.0,
               nb_hz: float = 0.0, nbursts: int = 0, burst_samples: int = 0,
               burst_amplitude: float = 0.0) -> None:
    """Seeded interference added in place to a device filterbank
    (psr_fb_inject_rfi): nb_channels narrowband channels modulated at nb_hz,
    and nbursts broadband bursts; amplitudes in sample units."""
    import ctypes as C

    from ._lib import check, lib

    class _R(C.Structure):
        _fields_ = [("seed", C.c_uint64), ("nb_channels", C.c_uint64),
                    ("nb_amplitude", C.c_double), ("nb_hz", C.c_double),
                    ("nbursts", C.c_uint64), ("burst_samples", C.c_uint64),
                    ("burst_amplitude", C.c_double)]

    r = _R(seed, nb_channels, nb_amplitude, nb_hz, nbursts, burst_samples, burst_amplitude)
    check(lib().psr_fb_inject_rfi(fb.handle, C.byref(r)))
