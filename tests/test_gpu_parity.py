"""GPU (libpsr through the C ABI) against the CPU oracle on seeded inputs.

Bit-exact: decoded samples, RFI masks and masked data, dedispersed series,
raw power spectra (the FFT is a fixed FP32 algorithm both sides implement),
per-trial candidate lists, fold bins/counts of integer-valued series.
Tolerances (written per test): profile statistics whose f64 sums are
reassociated (1e-12 relative)."""
import os

import numpy as np
import pytest

from test_oracle_golden import BIT_CASES, fixture, xorshift_train

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1


def c1_small(seed=11, ns=1 << 15, nch=32):
    from pulsarsr_gb300 import synth
    o = synth.config_c1(seed)
    o.nsamples, o.nchans, o.foff = ns, nch, -100.0 / nch
    return o


# ----------------------------------------------------------------- fbank
@pytest.mark.parametrize("bits,payload,expected", BIT_CASES)
def test_decode_bit_depth_fixtures(gpu, bits, payload, expected):
    from pulsarsr_gb300 import fbank
    fb = fbank.decode(fixture(bits, payload))
    assert fb.data.reshape(-1).tolist() == expected
    assert fbank.decode(fixture(bits, payload), 2).nsamples == 2


def test_decode_errors_match_reference_text(gpu, oracle):
    from pulsarsr_gb300 import FormatError, fbank
    bad = fixture(32, [0, 0, 128, 63, 0, 0, 0, 64, 0, 0, 128, 127, 0, 0, 0, 0])
    with pytest.raises(FormatError) as e:
        fbank.decode(bad)
    with pytest.raises(oracle.OracleError) as o:
        oracle.decode(bad)
    assert str(e.value) == str(o.value) == "invalid or unsupported filterbank: nonfinite sample at 1/0"
    with pytest.raises(FormatError, match="truncated frame"):
        fbank.decode(fixture(16, [1, 0, 2]))
    with pytest.raises(FormatError, match="need at least two samples"):
        fbank.decode(fixture(8, [1, 2]))


@pytest.mark.parametrize("nbits", [1, 2, 4, 8, 16, 32])
def test_decode_matches_oracle(gpu, oracle, nbits):
    from pulsarsr_gb300 import fbank, synth
    o = synth.Observation(nchans=40, nbits=nbits, nsamples=3000, tsamp=1e-4, fch1=1500.,
                          foff=-2.0, seed=nbits, noise_mean=(1 << min(nbits, 8)) / 2 if nbits < 32
                          else 10.0, noise_sigma=max((1 << min(nbits, 8)) / 6, 0.5))
    raw = o.to_bytes()
    fb = fbank.decode(raw)
    _, d = oracle.decode(raw)
    assert np.array_equal(fb.data, d)
    fb2 = fbank.decode(raw, 1234)
    assert np.array_equal(fb2.data, d[:, :1234])


# ------------------------------------------------------------------- rfi
@pytest.mark.parametrize("n", [0, 1, 2, 3, 10, 333, 1000, 65536, 100001])
def test_median_matches_oracle(gpu, oracle, n):
    from pulsarsr_gb300 import rfi
    rng = np.random.default_rng(n)
    v = rng.normal(0, 1, n).astype(np.float32)
    v[: n // 3] = np.round(v[: n // 3])  # ties, +0/-0
    if n > 5:
        v[1] = -0.0
        v[2] = 0.0
    m = rfi.median(v)
    o = oracle.median(v)
    assert np.float32(m).tobytes() == np.float32(o).tobytes()


def f32_filterbank(data, tsamp=1e-3, fch1=1400.0, foff=-1.0):
    from pulsarsr_gb300 import fbank, synth
    nch = data.shape[0]
    raw = synth.header_bytes(nch, 32, tsamp, fch1, foff) + synth.pack(data.T, 32)
    return fbank.decode(raw), raw


def test_rfi_reference_unit_cases(gpu, oracle):
    from pulsarsr_gb300 import rfi
    # rfi/src/lib.rs:101-114
    n, chans = 4000, 16
    i = np.arange(n * chans, dtype=np.uint64)
    data = (100. + ((i * np.uint64(2654435761)) % np.uint64(1000)).astype(np.float32) / 500. - 1.)
    data = data.astype(np.float32).reshape(chans, n)
    data[:, 1600:1680] += 30.
    fb, _ = f32_filterbank(data)
    m = rfi.mask(fb, 400, 8.)
    od, om = oracle.rfi_mask(data, 400, 8.)
    assert 4 in m.blocks
    assert (m.channels, m.blocks, m.masked_fraction) == (om["channels"], om["blocks"],
                                                          om["masked_fraction"])
    assert np.array_equal(fb.data, od)
    # rfi/src/lib.rs:116-129
    n = 1000
    data = (10. + (np.arange(n * 16) % 7)).astype(np.float32).reshape(16, n)
    data[0, :] = 1000.
    data[1:, 400:450] += 500.
    fb, _ = f32_filterbank(data)
    m = rfi.mask(fb, 50, 6.)
    od, om = oracle.rfi_mask(data, 50, 6.)
    assert 0 in m.channels and 8 in m.blocks and m.masked_fraction > 0.05
    assert (m.channels, m.blocks, m.masked_fraction) == (om["channels"], om["blocks"],
                                                          om["masked_fraction"])
    assert np.array_equal(fb.data, od)


@pytest.mark.parametrize("nbits,ns,block", [(8, 1 << 18, 1562), (4, 200000, 1388), (2, 50000, 400),
                                            (16, 40000, 999), (32, 30000, 777)])
def test_rfi_mask_matches_oracle(gpu, oracle, nbits, ns, block):
    from pulsarsr_gb300 import fbank, rfi, synth
    o = synth.Observation(nchans=48, nbits=nbits, nsamples=ns, tsamp=64e-6, fch1=1450.,
                          foff=-1.0, seed=100 + nbits,
                          noise_mean={2: 1.5, 4: 8., 8: 100., 16: 3000., 32: 100.}[nbits],
                          noise_sigma={2: 0.6, 4: 2., 8: 10., 16: 300., 32: 10.}[nbits],
                          gain_spread=0.2, bursts=3, burst_amplitude=4.0, burst_seconds=0.2)
    s = o.samples()
    hi = (1 << nbits) - 1 if nbits < 32 else None
    s[:, 5] = s[:, 5] // 2 if hi else s[:, 5] * 0.5  # a low channel
    s[:, 17] = hi if hi else 1e4                     # a saturated channel
    from pulsarsr_gb300.synth import pack
    raw = o.header() + pack(s, nbits)
    fb = fbank.decode(raw)
    m = rfi.mask(fb, block, 8.0)
    _, d = oracle.decode(raw)
    od, om = oracle.rfi_mask(d, block, 8.0)
    assert (m.channels, m.blocks) == (om["channels"], om["blocks"])
    assert m.masked_fraction == om["masked_fraction"]
    assert np.array_equal(fb.data, od)
    assert m.channels  # the planted channels are found


@pytest.mark.parametrize("case", ["c2", "u8_big_total", "u16", "dyadic_ties", "constant", "f32"])
def test_channel_stats_bit_exact(gpu, oracle, case):
    """rfi::mask's channel means and variances: the device's parallel
    reference-order sums against the oracle's sequential loops, bit for bit.
    u8_big_total: channel totals above 2^24, so the mean is an inexact f32
    chain too.  dyadic_ties: 2^16 samples of 0..3, so means and squared
    deviations have few bits and exact rounding ties occur as the sums grow."""
    from pulsarsr_gb300 import fbank, rfi, synth
    from pulsarsr_gb300.synth import pack
    rng = np.random.default_rng(7)
    if case == "c2":
        raw = synth.config_c2(2).to_bytes()
    else:
        nbits, ns = {"u8_big_total": (8, 1 << 20), "u16": (16, 60000),
                     "dyadic_ties": (8, 1 << 16), "constant": (8, 5000),
                     "f32": (32, 40000)}[case]
        o = synth.Observation(nchans=24, nbits=nbits, nsamples=ns, tsamp=64e-6, fch1=1450.,
                              foff=-1.0, seed=11, noise_mean=100., noise_sigma=10.)
        if case == "u8_big_total":
            x = np.clip(np.rint(rng.normal(200, 20, (ns, 24))), 0, 255)
        elif case == "u16":
            x = np.clip(np.rint(rng.normal(30000, 3000, (ns, 24))), 0, 65535)
        elif case == "f32":
            x = rng.normal(-3.0, 2.5, (ns, 24))
        elif case == "dyadic_ties":
            x = rng.integers(0, 4, (ns, 24)).astype(np.float64)
            x[:, 3] = 1.0
            x[::2, 4] = 3.0
            x[1::2, 4] = 0.0
        else:
            x = np.full((ns, 24), 7.0)
            x[:, 1] = 0.0
        raw = o.header() + pack(x.astype(np.float32), nbits)
    fb = fbank.decode(raw)
    m, v = rfi.channel_stats(fb)
    _, d = oracle.decode(raw)
    om, ov = oracle.channel_stats(d)
    assert m.tobytes() == om.tobytes()
    assert v.tobytes() == ov.tobytes()


# ------------------------------------------------------------ dedisperse
NOISE = {1: (0.5, 0.5), 2: (1.5, 1.0), 4: (8., 2.)}  # (mean, sigma) by bit depth; else (100, 10)


@pytest.mark.parametrize("nbits", [1, 2, 4, 8, 16, 32])
def test_dedisperse_matches_oracle(gpu, oracle, nbits):
    from pulsarsr_gb300 import dedisperse, fbank, synth
    mean, sigma = NOISE.get(nbits, (100., 10.))
    o = synth.Observation(nchans=96, nbits=nbits, nsamples=60000, tsamp=72e-6, fch1=1448.,
                          foff=-1.0, seed=7, noise_mean=mean, noise_sigma=sigma,
                          pulsars=[synth.Pulsar(0.0046214, 62.4, 0.03, 0.5)])
    raw = o.to_bytes()
    fb = fbank.decode(raw)
    _, d = oracle.decode(raw)
    freqs = fb.header.frequencies()
    for dm in (0.0, 10.0, 62.4, 499.9):
        dl = dedisperse.delays(freqs, o.tsamp, dm)
        a = dedisperse.apply(fb, dl)
        b = oracle.apply(d, dl)
        assert a.tobytes() == b.tobytes(), dm
        a = dedisperse.apply(fb, dl, 12345)
        assert a.tobytes() == oracle.apply(d, dl, 12345).tobytes()
    trials = dedisperse.plan(0, 300, dedisperse.dm_step(freqs, o.tsamp))[::7]
    n = 60000 - int(dedisperse.delays(freqs, o.tsamp, trials[-1]).max())
    out = dedisperse.apply_trials(fb, trials, n)
    for i in range(0, len(trials), 11):
        ref = oracle.apply(d, oracle.delays(freqs, o.tsamp, trials[i]), n)
        assert out[i].tobytes() == ref.tobytes(), i


@pytest.mark.parametrize("nbits,nch", [(8, 600), (4, 700)])
def test_dedisperse_many_channels(gpu, oracle, nbits, nch):
    """600 channels of 8-bit data: the packed kernel runs in channel groups of
    257 whose sums are added in f32 (exact below 2^24).  700 channels of 4-bit
    data: one group whose per-CTA delay block (8 trials x 700 channels) is too
    large to preload into shared memory, so stages read the delays from
    global memory."""
    from pulsarsr_gb300 import dedisperse, fbank, synth
    mean, sigma = NOISE.get(nbits, (120., 40.))
    o = synth.Observation(nchans=nch, nbits=nbits, nsamples=20000, tsamp=64e-6, fch1=1600.,
                          foff=-400.0 / nch, seed=12, noise_mean=mean, noise_sigma=sigma,
                          pulsars=[synth.Pulsar(0.0123, 150.0, 0.04, 0.5)])
    raw = o.to_bytes()
    fb = fbank.decode(raw)
    _, d = oracle.decode(raw)
    freqs = fb.header.frequencies()
    trials = dedisperse.plan(0, 100, dedisperse.dm_step(freqs, o.tsamp))[::5]
    n = 20000 - int(dedisperse.delays(freqs, o.tsamp, trials[-1]).max())
    out = dedisperse.apply_trials(fb, trials, n)
    for i in range(0, len(trials), 7):
        ref = oracle.apply(d, oracle.delays(freqs, o.tsamp, trials[i]), n)
        assert out[i].tobytes() == ref.tobytes(), i


@pytest.mark.parametrize("nbits", [4, 8])
def test_dedisperse_edge_shapes(gpu, oracle, nbits):
    """Unordered and repeated trial DMs in one launch, outputs of 2 samples and
    of one 4096-sample tile +- 1, and a single-channel observation."""
    from pulsarsr_gb300 import dedisperse, fbank, synth
    mean, sigma = NOISE.get(nbits, (100., 10.))
    o = synth.Observation(nchans=96, nbits=nbits, nsamples=12000, tsamp=72e-6, fch1=1448.,
                          foff=-1.0, seed=21, noise_mean=mean, noise_sigma=sigma)
    raw = o.to_bytes()
    fb = fbank.decode(raw)
    _, d = oracle.decode(raw)
    freqs = fb.header.frequencies()
    trials = np.array([300.0, 0.0, 150.0, 150.0, 7.25, 299.0, 0.5])
    for n in (2, 4095, 4096, 4097):
        out = dedisperse.apply_trials(fb, trials, n)
        for i, dm in enumerate(trials):
            ref = oracle.apply(d, oracle.delays(freqs, o.tsamp, dm), n)
            assert out[i].tobytes() == ref.tobytes(), (n, i)
    o1 = synth.Observation(nchans=1, nbits=nbits, nsamples=5000, tsamp=72e-6, fch1=1448.,
                           foff=-1.0, seed=22, noise_mean=mean, noise_sigma=sigma)
    raw1 = o1.to_bytes()
    fb1 = fbank.decode(raw1)
    _, d1 = oracle.decode(raw1)
    out = dedisperse.apply_trials(fb1, np.array([0.0, 100.0]), 4999)
    for i in range(2):
        assert out[i].tobytes() == d1[0, :4999].astype(np.float32).tobytes(), i


@pytest.mark.parametrize("subbands", [0, 4, 8])
@pytest.mark.parametrize("nbits,nch", [(4, 96), (8, 96), (8, 601), (2, 37)])
def test_dedisperse_subband_reuse_matches_oracle(gpu, oracle, subbands, nbits, nch):
    """Channel-by-channel and subband-reuse dedispersion (subbands of 4 or 8
    channels, each distinct intra-subband delay pattern of 8 consecutive
    trials summed once): bit-identical to the oracle for contiguous,
    fine-stepped trial DMs (where patterns repeat), a count that is not a
    multiple of 8, channel counts that are not multiples of the subband
    width, and 601 8-bit channels (three channel groups)."""
    from pulsarsr_gb300 import dedisperse, fbank, synth
    mean, sigma = NOISE.get(nbits, (100., 10.))
    o = synth.Observation(nchans=nch, nbits=nbits, nsamples=30000, tsamp=64e-6, fch1=1500.,
                          foff=-300.0 / nch, seed=40 + nbits, noise_mean=mean, noise_sigma=sigma,
                          pulsars=[synth.Pulsar(0.0123, 150.0, 0.04, 0.5)])
    raw = o.to_bytes()
    fb = fbank.decode(raw)
    _, d = oracle.decode(raw)
    freqs = fb.header.frequencies()
    plan = dedisperse.plan(0, 400, dedisperse.dm_step(freqs, o.tsamp))
    trials = np.concatenate([plan[100:145], plan[-21:]])
    n = 30000 - int(dedisperse.delays(freqs, o.tsamp, trials.max()).max())
    dedisperse.set_subbands(subbands)
    try:
        out, sums = dedisperse.apply_trials(fb, trials, n, with_sums=True)
    finally:
        dedisperse.set_subbands(-1)
    for i, dm in enumerate(trials):
        ref = oracle.apply(d, oracle.delays(freqs, o.tsamp, dm), n)
        assert out[i].tobytes() == ref.tobytes(), (subbands, i)
        assert sums[i] == float(np.add.accumulate(ref.astype(np.float64))[-1])


@pytest.mark.parametrize("subbands", [0, 4])
def test_search_subband_reuse_matches_oracle(gpu, oracle, subbands):
    """The GBT-shaped search's first 256 trial DMs with either dedispersion:
    candidate lists bit-identical to the oracle's."""
    from pulsarsr_gb300 import dedisperse, fbank, rfi, search, synth
    obs = synth.config_c2(2)
    raw, trials, disc = search_case(obs, 500.0)
    trials = trials[:256]
    cfg = dict(min_hz=15.0, max_hz=2000.0, threshold=8.0, max_candidates=32)
    block = max(int(0.1 / obs.tsamp), 32)
    fb = fbank.decode(raw)
    rfi.mask(fb, block, 8.0)
    dedisperse.set_subbands(subbands)
    try:
        counts, cands = search.search_trials(fb, trials, disc, search.Config(**cfg))
    finally:
        dedisperse.set_subbands(-1)
    _, d = oracle.decode(raw)
    md, _ = oracle.rfi_mask(d, block, 8.0)
    oc, ocands = oracle.search_trials(md, obs.frequencies(), obs.tsamp, trials, disc,
                                      threads=THREADS, **cfg)
    assert counts.tolist() == oc.tolist()
    assert cands.tobytes() == ocands.tobytes()


@pytest.mark.parametrize("nbits", [4, 8])
def test_stage_wait_gives_up_and_context_recovers(gpu, oracle, nbits):
    """The staged dedispersion kernel's bounded TMA waits: with its barriers
    armed and no copy issued (nothing in flight), every CTA gives up together
    and the host sees PSR_ETIMEOUT; the same context then dedisperses
    correctly.  f32 samples do not take the staged kernel."""
    from pulsarsr_gb300 import InvalidArgument, WaitTimeout, dedisperse, fbank, synth
    mean, sigma = NOISE.get(nbits, (100., 10.))
    o = synth.Observation(nchans=96, nbits=nbits, nsamples=12000, tsamp=72e-6, fch1=1448.,
                          foff=-1.0, seed=23, noise_mean=mean, noise_sigma=sigma)
    raw = o.to_bytes()
    fb = fbank.decode(raw)
    _, d = oracle.decode(raw)
    freqs = fb.header.frequencies()
    for _ in range(2):
        with pytest.raises(WaitTimeout, match="bounded wait for a staged tile gave up"):
            dedisperse.test_stage_timeout(fb, 1000)
        trials = np.array([0.0, 62.4, 150.0])
        out = dedisperse.apply_trials(fb, trials, 9000)
        for i, dm in enumerate(trials):
            assert out[i].tobytes() == oracle.apply(d, oracle.delays(freqs, o.tsamp, dm),
                                                    9000).tobytes()
    fbf, _ = f32_filterbank(np.ones((4, 100), dtype=np.float32))
    with pytest.raises(InvalidArgument, match="does not take the staged kernel"):
        dedisperse.test_stage_timeout(fbf, 1000)


def test_dedisperse_errors(gpu):
    from pulsarsr_gb300 import DedisperseError, dedisperse, fbank
    fb = fbank.decode(fixture(8, [1, 2, 3, 4]))
    with pytest.raises(DedisperseError, match="delay exceeds observation"):
        dedisperse.apply(fb, [3, 0])
    with pytest.raises(DedisperseError, match="invalid output length"):
        dedisperse.apply(fb, [0, 0], 3)


# ---------------------------------------------------------------- spectra
@pytest.mark.parametrize("n", [2, 3, 5, 16, 100, 1000, 4097, 8192, 8193, 130513, 263500])
def test_raw_power_bit_exact(gpu, oracle, n):
    from pulsarsr_gb300 import search
    rng = np.random.default_rng(n)
    for s in (rng.normal(0, 1, n).astype(np.float32),
              np.rint(rng.normal(800, 30, n)).astype(np.float32)):
        a = search.raw_power(s)
        b = oracle.raw_power(s)
        assert a.tobytes() == b.tobytes()


def test_periodicity_reference_cases(gpu, oracle):
    from pulsarsr_gb300 import search
    tsamp, f = 0.001, 31.25
    x = np.sin(2 * np.pi * f * np.arange(8192) * tsamp).astype(np.float32)
    c = search.periodicity(x, tsamp, 0., search.Config(min_hz=10.))
    assert abs(c[0]["frequency_hz"] - f) < 0.1
    assert c.tobytes() == oracle.periodicity(x, tsamp, 0., min_hz=10.).tobytes()
    c = search.periodicity(x, tsamp, 0., search.Config(min_hz=10., birdies=[(f, 1.)]))
    assert all(abs(c["frequency_hz"] - f) > 1.)
    assert c.tobytes() == oracle.periodicity(x, tsamp, 0., min_hz=10.,
                                             birdies=[(f, 1.)]).tobytes()
    dt, period, s = xorshift_train()
    c = search.periodicity(s, dt, 18.)
    assert c.tobytes() == oracle.periodicity(s, dt, 18.).tobytes()
    kept = search.sift(c, 1.5 / (s.size * dt), 10, False)
    assert abs(kept[0]["frequency_hz"] - 1. / period) < 0.2


@pytest.mark.parametrize("seed", range(4))
def test_periodicity_random_matches_oracle(gpu, oracle, seed):
    from pulsarsr_gb300 import search
    rng = np.random.default_rng(seed)
    n = int(rng.integers(20000, 140000))
    t = np.arange(n) * 64e-6
    x = rng.normal(0, 1, n) + 0.2 * (np.mod(t / 0.0123, 1.0) < 0.05)
    x = np.rint(40 * x + 500).astype(np.float32)
    cfg = dict(min_hz=5.0, max_hz=3000.0, threshold=6.0, max_candidates=int(rng.integers(8, 64)))
    c = search.periodicity(x, 64e-6, 3.0, search.Config(**cfg))
    o = oracle.periodicity(x, 64e-6, 3.0, **cfg)
    assert len(o) > 0
    assert c.tobytes() == o.tobytes()


@pytest.mark.parametrize("seed", range(3))
def test_periodicity_32_harmonics_matches_oracle(gpu, oracle, seed):
    """The h = 32 extension level: candidate lists bit-identical to the
    oracle's, with h = 32 entries present for a narrow pulse train."""
    from pulsarsr_gb300 import search
    from test_abi import harmonic_comb
    rng = np.random.default_rng(100 + seed)
    n = 1 << int(rng.integers(16, 19))
    x = harmonic_comb(rng, n, int(rng.integers(150, n // 160)))
    cfg = dict(min_hz=2.0, max_hz=3000.0, threshold=6.0, max_candidates=64, max_harmonics=32)
    c = search.periodicity(x, 64e-6, 3.0, search.Config(**cfg))
    o = oracle.periodicity(x, 64e-6, 3.0, **cfg)
    assert 32 in o["harmonics"].tolist()
    assert c.tobytes() == o.tobytes()
    # with birdies over a few of the comb's harmonics
    f0 = float(o["frequency_hz"][np.argmax(o["harmonics"])])
    cfg["birdies"] = [(f0 * 3, 0.5), (f0 * 17, 0.5)]
    c = search.periodicity(x, 64e-6, 3.0, search.Config(**cfg))
    o = oracle.periodicity(x, 64e-6, 3.0, **cfg)
    assert c.tobytes() == o.tobytes()


def search_case(obs, dm_max, ntake=None, rfi_on=True):
    from pulsarsr_gb300 import dedisperse, synth
    raw = obs.to_bytes()
    freqs = obs.frequencies()
    step = dedisperse.dm_step(freqs, obs.tsamp)
    trials = dedisperse.plan(0, dm_max, step)
    md = int(dedisperse.delays(freqs, obs.tsamp, dm_max).max())
    length = obs.nsamples - md
    discovery = (length - md) // 2
    if ntake:
        trials = trials[:: max(len(trials) // ntake, 1)]
    return raw, trials, discovery


@pytest.mark.parametrize("cfgname", ["c1", "c2", "c1h32"])
def test_search_trials_match_oracle(gpu, oracle, cfgname):
    """Candidate lists of the trial loop, GPU vs oracle, bit for bit, after
    the same RFI mask (the psr search path up to grouping)."""
    from pulsarsr_gb300 import fbank, rfi, search, synth
    if cfgname.startswith("c1"):
        obs = synth.config_c1(1)
        raw, trials, disc = search_case(obs, 120.0)
        trials = np.arange(0, 120.0 + 1e-9, 2.0)
        cfg = dict(min_hz=15.0, max_hz=2000.0, threshold=8.0, max_candidates=32)
        if cfgname == "c1h32":
            cfg["max_harmonics"] = 32
    else:
        obs = synth.config_c2(2)
        raw, trials, disc = search_case(obs, 500.0, ntake=64)
        cfg = dict(min_hz=15.0, max_hz=2000.0, threshold=8.0, max_candidates=32)
    block = max(int(0.1 / obs.tsamp), 32)
    fb = fbank.decode(raw)
    m = rfi.mask(fb, block, 8.0)
    counts, cands = search.search_trials(fb, trials, disc, search.Config(**cfg))
    _, d = oracle.decode(raw)
    md, om = oracle.rfi_mask(d, block, 8.0)
    assert (m.channels, m.blocks) == (om["channels"], om["blocks"])
    ocounts, ocands = oracle.search_trials(md, obs.frequencies(), obs.tsamp, trials, disc,
                                           threads=THREADS, **cfg)
    assert counts.tolist() == ocounts.tolist()
    assert cands.tobytes() == ocands.tobytes()
    assert counts.sum() > 0


def test_search_full_c2_every_trial(gpu, oracle):
    """Full 2000-trial GBT-shaped search on the GPU; the oracle recomputes
    every trial's list and all 2000 must match bit for bit."""
    from pulsarsr_gb300 import fbank, rfi, search, synth
    obs = synth.config_c2(2)
    raw, trials, disc = search_case(obs, 500.0)
    assert len(trials) == 2000
    cfg = dict(min_hz=15.0, max_hz=2000.0, threshold=8.0, max_candidates=32)
    fb = fbank.decode(raw)
    rfi.mask(fb, max(int(0.1 / obs.tsamp), 32), 8.0)
    counts, cands = search.search_trials(fb, trials, disc, search.Config(**cfg))
    starts = np.concatenate([[0], np.cumsum(counts)]).astype(int)
    _, d = oracle.decode(raw)
    md, _ = oracle.rfi_mask(d, max(int(0.1 / obs.tsamp), 32), 8.0)
    oc, ocands = oracle.search_trials(md, obs.frequencies(), obs.tsamp, trials, disc,
                                      threads=THREADS, **cfg)
    ostarts = np.concatenate([[0], np.cumsum(oc)]).astype(int)
    assert counts.tolist() == oc.tolist()
    for i in range(trials.size):
        a = cands[starts[i]:starts[i + 1]]
        b = ocands[ostarts[i]:ostarts[i + 1]]
        assert a.tobytes() == b.tobytes(), i
    # the injected 4.6214 ms pulsar is among the strongest candidates near DM 62.4
    near = cands[np.abs(cands["dm"] - 62.4) < 2.0]
    assert np.any(np.abs(near["frequency_hz"] - 1 / 0.0046214) < 0.05)


def test_injected_rfi_is_masked_like_the_oracle(gpu, oracle):
    """Seeded narrowband channels and broadband bursts added on the device
    (the survey workload's interference): the mask flags them, and mask,
    fraction and filled data equal the oracle's on the same samples."""
    from pulsarsr_gb300 import rfi, synth
    fb = synth.device(128, 8, 1 << 17, 64e-6, 1600.0, -400.0 / 128, seed=8, noise_mean=128.0,
                      noise_sigma=16.0, gain_spread=0.1)
    clean = fb.data
    synth.inject_rfi(fb, 8, nb_channels=3, nb_amplitude=48.0, nb_hz=50.0, nbursts=2,
                     burst_samples=781, burst_amplitude=32.0)
    d = fb.data
    changed = np.flatnonzero(np.any(d != clean, axis=1))
    nb = [c for c in changed if np.mean(d[c] != clean[c]) > 0.5]
    assert len(nb) == 3
    block = max(int(0.1 / 64e-6), 32)
    m = rfi.mask(fb, block, 8.0)
    od, om = oracle.rfi_mask(d, block, 8.0)
    assert set(nb) <= set(m.channels) and len(m.blocks) >= 2
    assert (m.channels, m.blocks, m.masked_fraction) == (om["channels"], om["blocks"],
                                                          om["masked_fraction"])
    assert np.array_equal(fb.data, od)


# --------------------------------------------------- f32-sample searches
def f32_obs(seed, noise_mean=100.0, nch=32, ns=1 << 16):
    """An f32 filterbank shaped like the reference's synthetic.fil (32 ch,
    65,536 samples at 250 us): non-integer samples, so the periodicity mean
    (a sequential f64 sum, search/src/lib.rs:36) is order-sensitive."""
    from pulsarsr_gb300 import synth
    return synth.Observation(nchans=nch, nbits=32, nsamples=ns, tsamp=2.5e-4, fch1=1500.0,
                             foff=-200.0 / nch, seed=seed, noise_mean=noise_mean,
                             noise_sigma=10.0 if noise_mean else 1.0,
                             pulsars=[synth.Pulsar(0.064, 40.0, 0.05, 0.6)])


def sequential_sum(x):
    """The reference's f64 series sum: one add after another, in order."""
    return float(np.add.accumulate(np.asarray(x, dtype=np.float64))[-1])


def test_f32_series_sums_are_the_sequential_sum(gpu):
    """Series sums on f32 samples equal the in-order f64 sum bit for bit,
    also where a reassociated sum would differ: a series whose small terms
    the sequential sum loses against a large one."""
    from pulsarsr_gb300 import dedisperse, fbank
    obs = f32_obs(31)
    fb = fbank.decode(obs.to_bytes())
    trials = np.arange(0.0, 120.0 + 1e-9, 8.0)
    n = 30000
    x, sums = dedisperse.apply_trials(fb, trials, n, with_sums=True)
    for i in range(trials.size):
        assert np.float64(sums[i]).tobytes() == np.float64(sequential_sum(x[i])).tobytes(), i
    # one channel, zero delay at every DM: the series is the channel itself
    y = np.full(5000, 2.0 ** -20, dtype=np.float32)
    y[1::3] *= np.float32(1.5)
    y[0], y[-1] = 2.0 ** 40, -(2.0 ** 40)
    fb1, _ = f32_filterbank(y[None, :])
    x1, s1 = dedisperse.apply_trials(fb1, np.array([0.0, 10.0]), y.size, with_sums=True)
    assert x1[0].tobytes() == y.tobytes()
    want = sequential_sum(y)
    assert want != float(np.sum(y.astype(np.float64)))  # pairwise differs here
    assert s1.tolist() == [want, want]


@pytest.mark.parametrize("noise_mean", [100.0, 0.0])
def test_search_trials_f32_match_oracle(gpu, oracle, noise_mean):
    """The trial loop on f32 samples, RFI on: candidate lists bit-identical
    to the oracle's (mean = the reference's sequential f64 sum)."""
    from pulsarsr_gb300 import fbank, rfi, search
    obs = f32_obs(32 if noise_mean else 33, noise_mean)
    raw = obs.to_bytes()
    trials = np.arange(0.0, 120.0 + 1e-9, 2.0)
    disc = 32000
    cfg = dict(min_hz=10.0, max_hz=2000.0, threshold=8.0, max_candidates=32)
    block = max(int(0.1 / obs.tsamp), 32)
    fb = fbank.decode(raw)
    m = rfi.mask(fb, block, 8.0)
    counts, cands = search.search_trials(fb, trials, disc, search.Config(**cfg))
    _, d = oracle.decode(raw)
    md, om = oracle.rfi_mask(d, block, 8.0)
    assert (m.channels, m.blocks) == (om["channels"], om["blocks"])
    oc, ocands = oracle.search_trials(md, obs.frequencies(), obs.tsamp, trials, disc,
                                      threads=THREADS, **cfg)
    assert counts.tolist() == oc.tolist()
    assert cands.tobytes() == ocands.tobytes()
    assert counts.sum() > 0


def test_session_f32_matches_oracle(gpu, oracle):
    """unpack -> RFI -> trial loop in a session on f32 samples, twice."""
    from pulsarsr_gb300 import fbank, search, session
    obs = f32_obs(34)
    raw = obs.to_bytes()
    hdr = fbank.parse_header(raw)
    trials = np.arange(0.0, 120.0 + 1e-9, 2.0)
    disc = 32000
    cfg = search.Config(min_hz=10.0, max_hz=2000.0, threshold=8.0)
    block = max(int(0.1 / obs.tsamp), 32)
    s = session.SearchSession(hdr, obs.nsamples, trials, disc, cfg, block, 8.0)
    _, d = oracle.decode(raw)
    md, om = oracle.rfi_mask(d, block, 8.0)
    oc, ocands = oracle.search_trials(md, obs.frequencies(), obs.tsamp, trials, disc,
                                      threads=THREADS, min_hz=10.0, max_hz=2000.0,
                                      threshold=8.0, max_candidates=32)
    for _ in range(2):
        s.load(raw[hdr.data_offset:])
        s.run()
        s.sync()
        counts, cands = s.candidates()
        assert counts.tolist() == oc.tolist()
        assert cands.tobytes() == ocands.tobytes()


def test_session_pipeline_matches_oracle(gpu, oracle):
    """unpack -> RFI -> trial loop in one device-resident session."""
    from pulsarsr_gb300 import fbank, search, session, synth
    obs = c1_small(seed=21)
    obs.nsamples = 1 << 16
    raw, trials, disc = search_case(obs, 120.0)
    hdr = fbank.parse_header(raw)
    cfg = search.Config(min_hz=15.0, max_hz=2000.0, threshold=8.0)
    block = max(int(0.1 / obs.tsamp), 32)
    s = session.SearchSession(hdr, obs.nsamples, trials, disc, cfg, block, 8.0)
    _, d = oracle.decode(raw)
    md, om = oracle.rfi_mask(d, block, 8.0)
    oc, ocands = oracle.search_trials(md, obs.frequencies(), obs.tsamp, trials, disc,
                                      threads=THREADS, min_hz=15.0, max_hz=2000.0,
                                      threshold=8.0, max_candidates=32)
    # Runs on the same buffers give the same answer, also with stage events
    # (1) and with the stages serialised for timing (2).
    for prof in (0, 1, 2):
        s.set_profiling(prof)
        s.stage_times(reset=True)
        s.load(raw[hdr.data_offset:])
        s.run()
        s.sync()
        st = s.stage_times()
        assert all(st[k][1] > 0 for k in ("dedisperse", "fft", "spectrum")) == (prof > 0)
        counts, cands = s.candidates()
        mask = s.mask()
        assert (mask["channels"], mask["blocks"]) == (om["channels"], om["blocks"])
        assert counts.tolist() == oc.tolist()
        assert cands.tobytes() == ocands.tobytes()
    with pytest.raises(Exception, match="0, 1 or 2"):
        s.set_profiling(3)


# ------------------------------------------------------------------- fold
def test_fold_matches_oracle(gpu, oracle):
    from pulsarsr_gb300 import dedisperse, fbank, fold, synth
    obs = synth.config_c1(3)
    obs.nsamples = 120000
    raw = obs.to_bytes()
    fb = fbank.decode(raw)
    x = dedisperse.apply(fb, dedisperse.delays(obs.frequencies(), obs.tsamp, 62.0))
    for period, bins, off in ((0.032, 64, 0), (0.0320011, 32, 0), (0.032, 128, 54321),
                              (0.00123456, 8, 7)):
        a = fold.profile_at(x, obs.tsamp, period, bins, off)
        b = oracle.profile_at(x, obs.tsamp, period, bins, off)
        assert a["bins"].tobytes() == b["bins"].tobytes()
        assert a["counts"].tolist() == b["counts"].tolist()
        assert a["snr"] == pytest.approx(b["snr"], rel=1e-12)
        assert a["reduced_chi_square"] == pytest.approx(b["reduced_chi_square"], rel=1e-12)
    r = fold.refine(x[:60000], obs.tsamp, 1 / 0.032, 1 / (60000 * obs.tsamp), 40, 64)
    o = oracle.refine(x[:60000], obs.tsamp, 1 / 0.032, 1 / (60000 * obs.tsamp), 40, 64)
    assert r["period_s"] == o["period_s"]
    assert r["bins"].tobytes() == o["bins"].tobytes()
    for start, width in ((13, 4), (60, 16), (0, 1)):
        a = fold.measure(x[5000:], 5000, obs.tsamp, 0.032, start, width, 64)
        b = oracle.measure(x[5000:], 5000, obs.tsamp, 0.032, start, width, 64)
        assert (a["on_samples"], a["off_samples"]) == (b["on_samples"], b["off_samples"])
        for k in ("snr", "mean_difference", "standard_error"):
            assert a[k] == pytest.approx(b[k], rel=1e-12, abs=1e-15)


def test_fold_reference_case(gpu):
    from pulsarsr_gb300 import fold
    i = np.arange(20000)
    x = np.where(i % 100 < 5, 10., ((i * 17 % 23) - 11.) / 10.).astype(np.float32)
    a = fold.profile(x, 0.001, 0.1, 32)
    b = fold.profile(x, 0.001, 0.1037, 32)
    assert a["snr"] > b["snr"] * 2 and int(a["counts"].sum()) == x.size
    i = np.arange(10000)
    within = ((i % 16) + 16 - 2) % 16 < 2
    y = np.where(within, 2., (i % 7) * 0.1).astype(np.float32)
    assert fold.measure(y[137:], 137, 0.001, 0.016, 2, 2, 16)["snr"] > 50.
    assert fold.measure(y[137:], 137, 0.001, 0.016, 10, 2, 16)["snr"] < 0.


def test_read_streams_file_like_decode(gpu, tmp_path):
    """fbank.read streams the payload in chunks; same samples as decode."""
    from pulsarsr_gb300 import IoError, fbank, synth
    o = synth.Observation(nchans=96, nbits=8, nsamples=1500000, tsamp=72e-6, fch1=1448.,
                          foff=-1.0, seed=21, noise_mean=100., noise_sigma=10.)
    raw = o.to_bytes()  # 144 MB payload: three 64 MiB chunks
    p = tmp_path / "x.fil"
    p.write_bytes(raw)
    a = fbank.read(str(p))
    b = fbank.decode(raw)
    assert a.nsamples == b.nsamples and a.data.tobytes() == b.data.tobytes()
    c = fbank.read(str(p), 12345)
    assert c.nsamples == 12345 and c.data.tobytes() == b.data[:, :12345].tobytes()
    with pytest.raises(IoError):
        fbank.read(str(tmp_path / "missing.fil"))
