"""Pin the CPU oracle against the reference: its unit-test literals and the
golden outputs it shipped (tests/golden/, extracted by make_golden.py)."""
import json
import math
import os
import struct

import numpy as np
import pytest

from conftest import GOLDEN, reference_file
from pulsarsr_gb300 import synth


def golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def fixture(bits, payload):
    """fbank/src/lib.rs:294-313: 2 channels, tsamp 1 ms, fch1 1400, foff -1."""
    b = synth._s("HEADER_START")
    for k, v in (("nchans", 2), ("nbits", bits), ("nifs", 1), ("data_type", 1)):
        b += synth._s(k) + struct.pack("<i", v)
    for k, v in (("tsamp", 0.001), ("fch1", 1400.0), ("foff", -1.0)):
        b += synth._s(k) + struct.pack("<d", v)
    return b + synth._s("HEADER_END") + bytes(payload)


BIT_CASES = [  # fbank/src/lib.rs:316-327
    (1, [0b10100110], [0., 1., 0., 0., 1., 0., 1., 1.]),
    (2, [0b11100100], [0., 2., 1., 3.]),
    (4, [0x21, 0x43], [1., 3., 2., 4.]),
    (8, [1, 2, 3, 4], [1., 3., 2., 4.]),
    (16, [1, 0, 2, 1, 3, 0, 4, 2], [1., 3., 258., 516.]),
    (32, [0, 0, 128, 63, 0, 0, 0, 64, 0, 0, 64, 64, 0, 0, 128, 64], [1., 3., 2., 4.]),
]


@pytest.mark.parametrize("bits,payload,expected", BIT_CASES)
def test_independent_bit_depth_fixtures(oracle, bits, payload, expected):
    _, d = oracle.decode(fixture(bits, payload))
    assert d.reshape(-1).tolist() == expected
    _, d2 = oracle.decode(fixture(bits, payload), 2)
    assert d2.shape[1] == 2


def test_decoder_rejections(oracle):
    with pytest.raises(oracle.OracleError, match="nonfinite"):
        oracle.decode(fixture(32, [0, 0, 128, 127] + [0] * 12))
    with pytest.raises(oracle.OracleError, match="truncated"):
        oracle.decode(fixture(16, [1, 0, 2]))
    b = synth._s("HEADER_START") + synth._s("surprise")
    with pytest.raises(oracle.OracleError, match="unknown keyword"):
        oracle.parse_header(b)


def test_roundtrip_preserves_channel_order(oracle):
    # fbank/src/lib.rs:260-280 with an independent f32 writer.
    data = np.array([[1., 2., 3.], [4., 5., 6.]], dtype=np.float32)
    raw = synth.header_bytes(2, 32, 0.001, 1400.0, -1.0) + synth.pack(data.T, 32)
    h, d = oracle.decode(raw)
    assert np.array_equal(d, data)
    with pytest.raises(oracle.OracleError):
        oracle.decode(raw[:-1])


def test_dedisperse_units_and_invalid_inputs(oracle):
    # dedisperse/src/lib.rs:109-115
    assert oracle.delays([1000., 2000.], 0.001, 1.).tolist() == [3, 0]
    with pytest.raises(oracle.OracleError):
        oracle.plan(0., 5., 0.)
    with pytest.raises(oracle.OracleError):
        oracle.delays([0.], 1., 1.)


@pytest.mark.parametrize("freqs", [[1400., 1300., 1200.], [1200., 1300., 1400.]])
def test_dispersed_delta_collapses(oracle, freqs):
    # dedisperse/src/lib.rs:95-108
    d = oracle.delays(freqs, 0.001, 20.)
    n = 100
    data = np.zeros((3, n), dtype=np.float32)
    for c, dl in enumerate(d):
        data[c, 10 + dl] = 1.
    out = oracle.apply(data, d)
    assert out[10] == 3. and out.sum() == 3.


def test_rfi_modest_broadband_burst(oracle):
    # rfi/src/lib.rs:101-114
    n, chans = 4000, 16
    i = np.arange(n * chans, dtype=np.uint64)
    data = (100. + ((i * np.uint64(2654435761)) % np.uint64(1000)).astype(np.float32) / 500. - 1.)
    data = data.astype(np.float32).reshape(chans, n)
    data[:, 1600:1680] += 30.
    _, m = oracle.rfi_mask(data, 400, 8.)
    assert 4 in m["blocks"]


def test_rfi_planted_channel_and_block(oracle):
    # rfi/src/lib.rs:116-129
    n = 1000
    data = (10. + (np.arange(n * 16) % 7)).astype(np.float32).reshape(16, n)
    data[0, :] = 1000.
    data[1:, 400:450] += 500.
    _, m = oracle.rfi_mask(data, 50, 6.)
    assert 0 in m["channels"] and 8 in m["blocks"] and m["masked_fraction"] > 0.05


def test_finds_sine_and_respects_birdies(oracle):
    # search/src/lib.rs:181-203
    tsamp, f = 0.001, 31.25
    x = np.sin(2 * np.pi * f * np.arange(8192) * tsamp).astype(np.float32)
    c = oracle.periodicity(x, tsamp, 0., min_hz=10.)
    assert abs(c[0]["frequency_hz"] - f) < 0.1
    c = oracle.periodicity(x, tsamp, 0., min_hz=10., birdies=[(f, 1.)])
    assert all(abs(c["frequency_hz"] - f) > 1.)


def test_sifts_dm_duplicates_and_harmonics(oracle):
    # search/src/lib.rs:205-226
    c = np.array([(100., .01, 20., 1, 10.), (200., .005, 21., 1, 8.), (100.01, .01, 19., 1, 9.),
                  (137., 1 / 137., 0., 1, 20.)], dtype=oracle.CAND_DTYPE)
    k = oracle.sift(c, 0.1, 10, True)
    assert len(k) == 1 and k[0]["dm"] == 20.


def xorshift_train():
    """search/src/lib.rs:229-243: off-bin Gaussian pulse train + xorshift noise."""
    dt, period = 0.00025, 0.02371
    state = 123456789
    out = np.empty(16384, dtype=np.float32)
    m = (1 << 64) - 1
    for i in range(16384):
        phase = math.modf(i * dt / period)[0]
        dist = abs(phase - 0.25)
        state ^= (state << 13) & m
        state ^= state >> 7
        state ^= (state << 17) & m
        noise = np.float32(state / float(m) - 0.5)
        out[i] = np.float32(math.exp(-0.5 * (dist / 0.013) ** 2)) + noise * np.float32(0.4)
    return dt, period, out


def test_off_bin_pulse_train_retains_fundamental(oracle):
    dt, period, s = xorshift_train()
    c = oracle.periodicity(s, dt, 18.)
    kept = oracle.sift(c, 1.5 / (s.size * dt), 10, False)
    assert abs(kept[0]["frequency_hz"] - 1. / period) < 0.2


def test_true_period_concentrates_pulses(oracle):
    # fold/src/lib.rs:350-364
    i = np.arange(20000)
    x = np.where(i % 100 < 5, 10., ((i * 17 % 23) - 11.) / 10.).astype(np.float32)
    a = oracle.profile_at(x, 0.001, 0.1, 32)
    b = oracle.profile_at(x, 0.001, 0.1037, 32)
    assert a["snr"] > b["snr"] * 2 and int(a["counts"].sum()) == x.size


def test_fixed_window_preserves_absolute_phase_and_sign(oracle):
    # search/src/confirmation.rs:544-572
    i = np.arange(10000)
    within = ((i % 16) + 16 - 2) % 16 < 2
    x = np.where(within, 2., (i % 7) * 0.1).astype(np.float32)
    a = oracle.measure(x[137:], 137, 0.001, 0.016, 2, 2, 16)
    assert a["snr"] > 50.
    b = oracle.measure(x[137:], 137, 0.001, 0.016, 10, 2, 16)
    assert b["snr"] < 0.


def test_fft_fp32_error_against_fp64(oracle):
    """The oracle's FP32 spectrum vs an FP64 FFT of the same input: norm-wise
    relative error below 1e-5 (the stated spectrum tolerance)."""
    rng = np.random.default_rng(5)
    s = np.rint(rng.normal(800, 30, 130513)).astype(np.float32)
    p32 = oracle.raw_power(s).astype(np.float64)
    p64 = oracle.raw_power_f64(s)
    rel = np.linalg.norm(p32 - p64) / np.linalg.norm(p64)
    assert rel < 1e-5, rel


# ---------------------------------------------------------- golden files
def test_gbt_dm62_delays_and_series_length(oracle):
    g = golden("gbt_dm62_series.json")
    raw = open(reference_file("GBT_Lband_PSR.fil"), "rb").read()
    h, d = oracle.decode(raw)
    freqs = h["fch1"] + np.arange(h["nchans"]) * h["foff"]
    dl = oracle.delays(freqs, h["tsamp"], g["dm"])
    assert dl.tolist() == g["delays"]
    assert oracle.apply(d, dl).size == g["samples"]


def test_gbt_fold_is_bit_exact(oracle):
    g = golden("gbt_fold.json")
    raw = open(reference_file("GBT_Lband_PSR.fil"), "rb").read()
    h, d = oracle.decode(raw)
    freqs = h["fch1"] + np.arange(h["nchans"]) * h["foff"]
    x = oracle.apply(d, oracle.delays(freqs, h["tsamp"], g["dm"]))
    p = oracle.profile_at(x, h["tsamp"], g["profile"]["period_s"], len(g["profile"]["bins"]))
    assert np.array_equal(p["bins"], np.array(g["profile"]["bins"], dtype=np.float32))
    assert p["counts"].tolist() == g["profile"]["counts"]
    assert p["snr"] == g["profile"]["snr"]
    assert p["reduced_chi_square"] == g["profile"]["reduced_chi_square"]


def test_gbt_rfi_mask_is_exact(oracle):
    g = golden("gbt_report_summary.json")["rfi"]
    raw = open(reference_file("GBT_Lband_PSR.fil"), "rb").read()
    h, d = oracle.decode(raw)
    _, m = oracle.rfi_mask(d, g["block_samples"], 8.0)
    assert m["channels"] == g["channels"] and m["blocks"] == g["blocks"]
    assert m["masked_fraction"] == g["masked_fraction"]


def compare_report(o, g, score_rtol):
    oc = o["confirmation"]
    for k, v in g["confirmation"].items():
        assert oc[k] == v, k
    assert o["rfi"]["channels"] == g["rfi"]["channels"]
    assert o["rfi"]["blocks"] == g["rfi"]["blocks"]
    assert len(oc["candidates"]) == len(g["families"])
    for a, b in zip(oc["candidates"], g["families"]):
        ca = a["candidate"]
        assert (ca["dm"], ca["harmonics"]) == (b["candidate"][1], b["candidate"][2])
        assert ca["score"] == pytest.approx(b["candidate"][3], rel=score_rtol)
        assert ca["frequency_hz"] == pytest.approx(b["candidate"][0], rel=1e-9)
        assert a["refined_dm"] == b["refined_dm"]
        assert a["window"] == b["window"] and a["zero_dm_window"] == b["zero_dm_window"]
        assert a["accepted"] == b["accepted"]
        assert a["rejection_reasons"] == b["rejection_reasons"]
        # members: same (dm, harmonics, frequency) set, scores within tolerance
        ma = sorted((m["dm"], m["harmonics"], m["frequency_hz"], m["score"])
                    for m in a["harmonic_members"])
        mb = sorted((m[1], m[2], m[0], m[3]) for m in b["harmonic_members"])
        assert len(ma) == len(mb)
        for x, y in zip(ma, mb):
            assert x[0] == y[0] and x[1] == y[1]
            assert x[2] == pytest.approx(y[2], rel=1e-9)
            assert x[3] == pytest.approx(y[3], rel=score_rtol)
        for key in ("validation", "zero_dm_validation"):
            for f in ("snr", "mean_difference", "standard_error"):
                assert a[key][f] == pytest.approx(b[key][f], rel=1e-9, abs=1e-12)
        assert np.allclose(a["profile"]["bins"], b["profile"]["bins"], rtol=1e-7)


def test_synthetic_search_matches_reference_report(oracle):
    g = golden("synth_report_summary.json")
    raw = open(reference_file("synthetic.fil"), "rb").read()
    o = oracle.psr_search(raw, dm_min=0, dm_max=120, dm_step=2.0, min_hz=10, max_hz=2000,
                          threshold=8, top=5, bins=64, threads=os.cpu_count() or 1)
    compare_report(o, g, score_rtol=2e-6)


@pytest.mark.slow
def test_gbt_search_matches_reference_report(oracle):
    """The full 2000-trial GBT search (cli/src/main.rs:380-571): every family,
    member, window and measurement of output_confirm_gbt/report.json."""
    g = golden("gbt_report_summary.json")
    raw = open(reference_file("GBT_Lband_PSR.fil"), "rb").read()
    o = oracle.psr_search(raw, dm_min=0, dm_max=500, min_hz=15, max_hz=2000, threshold=8,
                          top=5, bins=64, threads=os.cpu_count() or 1)
    assert o["trial_count"] == g["settings"]["trial_count"]
    assert o["dm_step"] == g["settings"]["dm_step"]
    compare_report(o, g, score_rtol=2e-6)
