"""Batched search of observations of uneven shape through one CUDA graph
launch: every observation's candidates equal those of its own search and
the oracle's."""
import os

import numpy as np
import pytest

THREADS = os.cpu_count() or 1

SHAPES = [  # (nchans, nsamples, tsamp, fch1, foff, dm_max, period, dm)
    (64, 1 << 16, 64e-6, 1450.0, -1.5625, 120.0, 0.032, 62.0),
    (128, 90000, 128e-6, 1500.0, -2.0, 300.0, 0.0523, 150.0),
    (96, 1 << 17, 100e-6, 1400.0, -1.0, 80.0, 0.0117, 33.0),
    (200, 70000, 256e-6, 1500.0, -1.5, 500.0, 0.31, 250.0),
    (64, 50000, 64e-6, 1450.0, -1.5625, 60.0, 0.0021, 20.0),
]


def observation(i):
    from pulsarsr_gb300 import synth
    nch, ns, tsamp, fch1, foff, _, P, DM = SHAPES[i]
    return synth.Observation(nchans=nch, nbits=8, nsamples=ns, tsamp=tsamp, fch1=fch1,
                             foff=foff, seed=100 + i, noise_mean=100.0, noise_sigma=10.0,
                             pulsars=[synth.Pulsar(P, DM, 0.05, 0.6)])


def plan(i, freqs, tsamp):
    from pulsarsr_gb300 import dedisperse
    dm_max = SHAPES[i][5]
    trials = dedisperse.plan(0.0, dm_max, 4 * dedisperse.dm_step(freqs, tsamp))
    md = int(dedisperse.delays(freqs, tsamp, dm_max).max())
    ns = SHAPES[i][1]
    return trials, (ns - 2 * md) // 2


@pytest.mark.gpu
def test_batch_graph_equals_individual_searches(gpu, oracle):
    from pulsarsr_gb300 import batch, fbank, rfi, search
    cfg = search.Config(min_hz=1.0, max_hz=2000.0, threshold=8.0, max_candidates=32)
    obs, raws, want = [], [], []
    for i in range(len(SHAPES)):
        o = observation(i)
        raw = o.to_bytes()
        h = fbank.parse_header(raw)
        trials, disc = plan(i, h.frequencies(), h.tsamp)
        block = max(int(0.1 / h.tsamp), 32)
        obs.append(dict(header=h, nsamples=o.nsamples, trials=trials, discovery=disc,
                        config=cfg, rfi_block=block, rfi_threshold=8.0))
        raws.append(np.frombuffer(raw, dtype=np.uint8)[h.data_offset:].copy())
        fb = fbank.decode(raw)
        rfi.mask(fb, block, 8.0)
        want.append(search.search_trials(fb, trials, disc, cfg))
        # the individual search against the oracle (RFI mask, then every trial)
        _, d = oracle.decode(raw)
        md, _ = oracle.rfi_mask(d, block, 8.0)
        oc, ocands = oracle.search_trials(md, h.frequencies(), h.tsamp, trials, disc,
                                          threads=THREADS, min_hz=1.0, max_hz=2000.0,
                                          threshold=8.0, max_candidates=32)
        assert np.array_equal(want[i][0], oc), i
        assert want[i][1].tobytes() == ocands.tobytes(), i
    b = batch.Batch(obs, hbm_budget_bytes=1 << 28)  # small budget: several DM blocks
    for i, p in enumerate(raws):
        b.load(i, p)
    for rnd in range(4):
        if rnd == 2:
            b.tune()
        if rnd == 3:
            # odd blocks and FFT launches smaller than a block: several launch
            # pairs per block, both halves of the spectra buffers, a short
            # last block
            for i in range(len(SHAPES)):
                b.set_chunking(i, 23, 5 + i)
        b.run()
        b.sync()
        for i in range(len(SHAPES)):
            c, x = b.candidates(i)
            assert np.array_equal(c, want[i][0]), (rnd, i)
            assert x.tobytes() == want[i][1].tobytes(), (rnd, i)


@pytest.mark.gpu
def test_batch_loads_device_generated_observations(gpu):
    from pulsarsr_gb300 import batch, fbank, rfi, search, synth
    cfg = search.Config(min_hz=1.0, max_hz=2000.0, threshold=8.0, max_candidates=32)
    fbs, obs = [], []
    for i in (0, 1):
        nch, ns, tsamp, fch1, foff, _, P, DM = SHAPES[i]
        fb = synth.device(nch, 8, ns, tsamp, fch1, foff, seed=7 + i, noise_mean=100.0,
                          noise_sigma=10.0, pulsars=[synth.Pulsar(P, DM, 0.05, 0.6)])
        trials, disc = plan(i, fb.header.frequencies(), tsamp)
        h = fbank.HeaderInfo(nch, 8, tsamp, fch1, foff, 0)
        obs.append(dict(header=h, nsamples=ns, trials=trials, discovery=disc, config=cfg,
                        rfi_block=0))
        fbs.append((fb, trials, disc))
    b = batch.Batch(obs)
    for i, (fb, _, _) in enumerate(fbs):
        b.load_fb(i, fb)
    b.run()
    b.sync()
    for i, (fb, trials, disc) in enumerate(fbs):
        c, x = b.candidates(i)
        c2, x2 = search.search_trials(fb, trials, disc, cfg)
        assert np.array_equal(c, c2) and x.tobytes() == x2.tobytes()
