"""The survey-scale search at its full shape: 4096 channels x 8-bit x 2^23
samples at 64 us (1200-1600 MHz), 8000 trials over DM 0-3000, rFFT 2^23 and
harmonic sums to 32.  Eight trial DMs spread over the plan (the first and
the last included) are searched on the GPU and recomputed by the oracle:
the candidate lists must be identical bit for bit.

The 34 GB observation is generated in HBM; the oracle's dedispersed series
are built from 128-channel slices copied to the host, adding the slices'
channel-ordered f32 sums in channel order (exact: every partial sum is an
integer below 4096 * 255 < 2^24, as in the reference's own loop,
dedisperse/src/lib.rs:80-88)."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def survey_pulsars(seed=5):
    from pulsarsr_gb300 import synth
    rng = np.random.default_rng(seed)
    return [synth.Pulsar(float(np.exp(rng.uniform(np.log(0.001), np.log(4.0)))),
                         float(rng.uniform(5, 2500)), float(rng.uniform(0.02, 0.06)),
                         float(rng.uniform(0.01, 0.04)), phase=float(rng.uniform(0, 1)))
            for _ in range(20)]


def test_survey_shape_trials_match_oracle(gpu, oracle):
    from pulsarsr_gb300 import dedisperse, search, synth
    nch, ns, tsamp, fch1, foff = 4096, 1 << 23, 64e-6, 1600.0, -400.0 / 4096
    fb = synth.device(nch, 8, ns, tsamp, fch1, foff, seed=5, noise_mean=128.0,
                      noise_sigma=16.0, gain_spread=0.1, pulsars=survey_pulsars())
    freqs = fb.header.frequencies()
    plan = dedisperse.plan(0.0, 3000.0, 0.37504)
    assert plan.size == 8000
    md = int(dedisperse.delays(freqs, tsamp, plan[-1]).max())
    disc = (ns - 2 * md) // 2
    pick = plan[np.linspace(0, plan.size - 1, 8).round().astype(int)]
    cfg = dict(min_hz=15.0, max_hz=2000.0, threshold=8.0, max_candidates=32, max_harmonics=32)
    counts, cands = search.search_trials(fb, pick, disc, search.Config(**cfg))

    dl = [oracle.delays(freqs, tsamp, dm) for dm in pick]
    series = np.zeros((pick.size, disc), dtype=np.float32)
    step = 128
    with ThreadPoolExecutor(pick.size) as pool:
        for c0 in range(0, nch, step):
            blk = fb.channels(c0, step)
            parts = list(pool.map(lambda i: oracle.apply(blk, dl[i][c0:c0 + step], disc),
                                  range(pick.size)))
            for i in range(pick.size):
                series[i] += parts[i]
        lists = list(pool.map(lambda i: oracle.periodicity(series[i], tsamp, pick[i], **cfg),
                              range(pick.size)))
    assert counts.tolist() == [len(x) for x in lists]
    assert cands.tobytes() == np.concatenate(lists).tobytes()
    assert counts.sum() > 0
