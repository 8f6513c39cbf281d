"""C ABI checks that need no GPU: the library builds, loads and exports every
function include/psr.h declares; host-side functions match the oracle."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    text = open(os.path.join(ROOT, "include", "psr.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(psr_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def L():
    from pulsarsr_gb300 import build
    build.build()
    from pulsarsr_gb300 import _lib
    return _lib.lib()


def test_exports_every_declared_symbol(L):
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_version(L):
    import pulsarsr_gb300
    assert "sm_103a" in pulsarsr_gb300.version()


def test_parse_header_matches_oracle_and_errors(L, oracle):
    from pulsarsr_gb300 import FormatError, IoError, fbank, synth
    raw = synth.header_bytes(96, 4, 7.2e-5, 1448.0, -1.0) + bytes(96 // 2 * 4)
    h = fbank.parse_header(raw)
    o = oracle.parse_header(raw)
    assert (h.nchans, h.nbits, h.tsamp, h.fch1, h.foff, h.data_offset) == \
        (o["nchans"], o["nbits"], o["tsamp"], o["fch1"], o["foff"], o["data_offset"])
    with pytest.raises(FormatError, match="unknown keyword surprise"):
        fbank.parse_header(synth._s("HEADER_START") + synth._s("surprise"))
    with pytest.raises(FormatError, match="missing HEADER_START"):
        fbank.parse_header(synth._s("HEADER_BEGIN"))
    with pytest.raises(IoError):
        fbank.parse_header(synth._s("HEADER_START")[:-2])


@pytest.mark.parametrize("dm", [0.0, 0.25, 62.0, 62.389, 499.86, 3000.0])
def test_delays_match_oracle(L, oracle, dm):
    from pulsarsr_gb300 import dedisperse
    for freqs, tsamp in ((1447.5 - np.arange(96), 7.2e-5), (1450 - 1.5625 * np.arange(64), 64e-6),
                         (1200 + np.arange(4096) * (400 / 4096), 64e-6)):
        assert np.array_equal(dedisperse.delays(freqs, tsamp, dm), oracle.delays(freqs, tsamp, dm))


def test_plan_and_step_match_oracle(L, oracle):
    from pulsarsr_gb300 import DedisperseError, dedisperse
    f = 1447.5 - np.arange(96)
    assert dedisperse.dm_step(f, 7.2e-5) == oracle.dm_step(f, 7.2e-5)
    step = dedisperse.dm_step(f, 7.2e-5)
    assert np.array_equal(dedisperse.plan(0, 500, step), oracle.plan(0, 500, step))
    assert dedisperse.delays([1000., 2000.], 0.001, 1.).tolist() == [3, 0]
    with pytest.raises(DedisperseError, match="invalid DM bounds/step"):
        dedisperse.plan(0., 5., 0.)
    with pytest.raises(DedisperseError, match="positive frequencies"):
        dedisperse.delays([0.], 1., 1.)
    with pytest.raises(DedisperseError, match="more than 100000"):
        dedisperse.plan(0., 1e6, 1.)


def test_sift_matches_oracle(L, oracle):
    from pulsarsr_gb300 import search
    rng = np.random.default_rng(7)
    n = 400
    c = np.zeros(n, dtype=search.CAND_DTYPE)
    c["frequency_hz"] = rng.choice([10.0, 20.0, 30.0, 47.3, 100.0], n) + rng.normal(0, 0.01, n)
    c["period_s"] = 1 / c["frequency_hz"]
    c["dm"] = rng.choice([0.0, 5.0, 62.0], n)
    c["harmonics"] = rng.choice([1, 2, 4], n)
    c["score"] = np.round(rng.normal(10, 3, n), 1)  # ties exercise the stable order
    for reject in (False, True):
        a = search.sift(c, 0.02, 7, reject)
        b = oracle.sift(c, 0.02, 7, reject)
        assert a.tobytes() == b.tobytes()
    c2 = np.array([(100., .01, 20., 1, 10.), (200., .005, 21., 1, 8.), (100.01, .01, 19., 1, 9.),
                   (137., 1 / 137., 0., 1, 20.)], dtype=search.CAND_DTYPE)
    k = search.sift(c2, 0.1, 10, True)
    assert len(k) == 1 and k[0]["dm"] == 20.


def harmonic_comb(rng, n, cycles):
    """32 equal harmonics of `cycles` cycles per n samples in weak noise: a
    high S/N comb whose parabolic bin offsets are accurate enough for the
    h = 32 sum to win."""
    t = np.arange(n)
    x = rng.normal(0, 0.1, n)
    for j in range(1, 33):
        x += 0.05 * np.cos(2 * np.pi * j * cycles * t / n + rng.uniform(0, 2 * np.pi))
    return np.rint(40 * x + 500).astype(np.float32)


def test_max_harmonics_levels(L, oracle):
    """max_harmonics 0/16 keeps the reference's levels; 32 adds h = 32 (the
    oracle's lists gain h = 32 entries for a narrow pulse); other values are
    rejected by the library before any device work."""
    from pulsarsr_gb300 import InvalidArgument, search
    x = harmonic_comb(np.random.default_rng(11), 1 << 16, 300)
    ref = oracle.periodicity(x, 1e-3, 0.0, min_hz=0.5, threshold=6.0, max_candidates=64)
    assert ref.tobytes() == oracle.periodicity(x, 1e-3, 0.0, min_hz=0.5, threshold=6.0,
                                               max_candidates=64, max_harmonics=16).tobytes()
    ext = oracle.periodicity(x, 1e-3, 0.0, min_hz=0.5, threshold=6.0, max_candidates=64,
                             max_harmonics=32)
    assert set(ref["harmonics"].tolist()) <= {1, 2, 4, 8, 16}
    assert 32 in ext["harmonics"].tolist()
    assert ext["score"].max() >= ref["score"].max()
    for bad in (1, 8, 24, 64):
        with pytest.raises(InvalidArgument, match="valid config"):
            search.periodicity(x, 1e-3, 0.0, search.Config(max_harmonics=bad))


def test_batch_and_stats_reject_bad_arguments(L):
    """Argument checks that run before any device work."""
    import ctypes as C
    from pulsarsr_gb300 import _lib
    assert L.psr_batch_set_chunking(None, C.c_uint64(0), C.c_uint64(16), C.c_uint64(0)) == \
        _lib.PSR_EINVAL
    assert L.psr_channel_stats(None, None, None) == _lib.PSR_EINVAL


def test_harmonic_division_gate_bound():
    """The harmonic-item kernel skips the correctly rounded division
    (sum - h) / RN(sqrt(h)) for h = 2, 8, 32 when x * RN(1/sqrt(2)) / 2^k is
    below thr - |thr| 2^-49.  Check on IEEE doubles that such a quotient is
    always below thr, and that the gap between the two is within 2^-50."""
    rng = np.random.default_rng(3)
    r1 = 0.7071067811865476
    for hi, c in ((1, 1.4142135623730951), (3, 2.8284271247461903), (5, 5.656854249492381)):
        assert c == np.sqrt(np.float64(1 << hi))
        r = r1 * 2.0 ** (-(hi >> 1))
        x = np.concatenate([rng.uniform(-50, 400, 400000),
                            np.exp(rng.uniform(-700, 700, 200000)),
                            -np.exp(rng.uniform(-700, 700, 50000))])
        q = x / c
        a = x * r
        nz = q != 0
        assert np.all(np.abs(a[nz] - q[nz]) <= np.abs(q[nz]) * 2.0 ** -50)
        for thr in (8.0, 0.5, 1e-300, -3.0, 0.0):
            skip = a < thr - abs(thr) * 2.0 ** -49
            assert not np.any(q[skip] >= thr), (hi, thr)
        # quotients straddling the threshold: x chosen so that x / c is within
        # a few ulps of 8
        xs = 8.0 * c * (1.0 + rng.integers(-40, 41, 100000) * 2.0 ** -52)
        qs, as_ = xs / c, xs * r
        skip = as_ < 8.0 - 8.0 * 2.0 ** -49
        assert not np.any(qs[skip] >= 8.0)
