"""Gradient refinement of (P, Pdot, DM): the adjoint against finite
differences and the FP64 oracle gradient, and the refined parameters against
the injected truth and the reference's grid refinement."""
import numpy as np
import pytest

# A 64-channel f32 filterbank, 1100-1500 MHz, 64 us, 2^17 samples (8.4 s),
# with one 23.7 ms pulsar at DM 71.3.
NCH, NS, TSAMP, FCH1, FOFF = 64, 1 << 17, 64e-6, 1500.0, -400.0 / 64
TRUE_P, TRUE_DM, TRUE_PDOT = 0.0237, 71.3, 0.0
N = NS - 4096


def observation(seed=4, amplitude=0.6):
    from pulsarsr_gb300 import synth
    return synth.Observation(nchans=NCH, nbits=32, nsamples=NS, tsamp=TSAMP, fch1=FCH1,
                             foff=FOFF, seed=seed, noise_mean=0.0, noise_sigma=1.0,
                             pulsars=[synth.Pulsar(TRUE_P, TRUE_DM, 0.05, amplitude)],
                             name="refine test")


@pytest.fixture(scope="module")
def obs_data():
    o = observation()
    x = o.samples()  # (ns, nch) f32
    return o, np.ascontiguousarray(x.T)


def mid_epoch(t, T):
    """Period at the middle of a span of T seconds (P and Pdot at the start are
    nearly degenerate over short spans; the mid-span period is not)."""
    t = t.copy()
    t["period_s"] = t["period_s"] + t["pdot"] * T / 2
    return t


def central(f, x, h):
    return (f(x + h) - f(x - h)) / (2 * h)


# Finite-difference steps.  DM: 1e-6 relative.  P and Pdot: steps that move
# the last sample's phase by ~1e-5 bins.  The cloud-in-cell objective is
# piecewise quadratic, with a kink wherever a sample crosses a bin edge; a
# 1e-6 relative step in P moves the last sample by 0.04 bins here (0.1-0.4
# cycles at 2^23 samples), so its secant is not the derivative.
H_P, H_PDOT, H_DM = 1e-10, 1e-12, 1e-6


def test_oracle_gradient_matches_finite_differences(obs_data, oracle):
    """The FP64 adjoint formulas against central differences."""
    o, data = obs_data
    freqs = o.frequencies()
    P, D = TRUE_P * (1 + 3e-6), TRUE_DM + 0.4

    def J(p, pd, d):
        return oracle.refine_objective(data, freqs, TSAMP, N, p, pd, d, 128, 64,
                                       variance=vfix)[0]
    # hold the variance fixed at the evaluation point, as the model does
    vfix = float(np.var(_y64(data, freqs, D)))
    J0, g, _ = oracle.refine_objective(data, freqs, TSAMP, N, P, 0.0, D, 128, 64, variance=vfix)
    fd_p = central(lambda x: J(x, 0.0, D), P, P * H_P)
    fd_d = central(lambda x: J(P, 0.0, x), D, D * H_DM)
    fd_pd = central(lambda x: J(P, x, D), 0.0, H_PDOT)
    assert np.isclose(g[0], fd_p, rtol=1e-4), (g[0], fd_p)
    assert np.isclose(g[2], fd_d, rtol=1e-4), (g[2], fd_d)
    assert np.isclose(g[1], fd_pd, rtol=1e-3), (g[1], fd_pd)


def _y64(data, freqs, dm):
    k = 4148.808 * (1 / freqs ** 2 - 1 / freqs.max() ** 2) / TSAMP
    tau = k * dm
    m = np.floor(tau).astype(int)
    a = tau - m
    y = np.zeros(N)
    for c in range(len(freqs)):
        row = data[c].astype(np.float64)
        y += (1 - a[c]) * row[m[c]:m[c] + N] + a[c] * row[m[c] + 1:m[c] + 1 + N]
    return y


@pytest.mark.gpu
def test_device_objective_and_adjoint_match_fp64(gpu, oracle, obs_data):
    from pulsarsr_gb300 import fbank, fold
    o, data = obs_data
    fb = fbank.decode(o.to_bytes())
    freqs = o.frequencies()
    for P, D, PD in ((TRUE_P, TRUE_DM, 0.0), (TRUE_P * (1 + 4e-6), TRUE_DM - 0.7, 1e-9),
                     (TRUE_P * (1 - 2e-6), TRUE_DM + 1.1, -3e-10)):
        vfix = float(np.var(_y64(data, freqs, D)))
        Jd, gd, pd, cells = fold.refine_objective(fb, N, P, PD, D, 128, 64, variance=vfix)
        Jo, go, po = oracle.refine_objective(data, freqs, TSAMP, N, P, PD, D, 128, 64,
                                             variance=vfix)
        # The device sums 64 channels per sample in f32 (about 2^-24 relative
        # each) and accumulates cells and adjoint terms in f64: measured on a
        # GB300, J within 6e-9 and every gradient component within 2e-6 of
        # the FP64 oracle; the bounds leave a 10x margin.
        assert np.isclose(Jd, Jo, rtol=1e-7), (Jd, Jo)
        assert np.allclose(pd, po, rtol=1e-4, atol=1e-3 * np.abs(po).max())
        assert np.allclose(cells.sum(axis=0), pd, rtol=1e-9, atol=1e-6)
        assert np.allclose(gd, go, rtol=2e-5, atol=1e-7 * np.abs(go).max()), (gd, go)


@pytest.mark.gpu
def test_device_adjoint_matches_finite_differences(gpu, obs_data):
    from pulsarsr_gb300 import fbank, fold
    o, data = obs_data
    fb = fbank.decode(o.to_bytes())
    P, D = TRUE_P * (1 + 3e-6), TRUE_DM + 0.4
    vfix = 1.0

    def J(p, pd, d):
        return fold.refine_objective(fb, N, p, pd, d, 128, 64, variance=vfix)[0]
    _, g, _, _ = fold.refine_objective(fb, N, P, 0.0, D, 128, 64, variance=vfix)
    assert np.isclose(g[0], central(lambda x: J(x, 0.0, D), P, P * H_P), rtol=1e-3)
    assert np.isclose(g[2], central(lambda x: J(P, 0.0, x), D, D * H_DM), rtol=5e-3)
    assert np.isclose(g[1], central(lambda x: J(P, x, D), 0.0, H_PDOT), rtol=1e-3)


@pytest.mark.gpu
def test_gradient_refinement_reaches_truth_and_grid(gpu, obs_data):
    from pulsarsr_gb300 import dedisperse, fbank, fold
    o, data = obs_data
    fb = fbank.decode(o.to_bytes())
    freqs = o.frequencies()
    T = N * TSAMP
    resolution = 1.0 / T
    step = dedisperse.dm_step(freqs, TSAMP)
    rng = np.random.default_rng(7)
    starts = []
    for _ in range(8):
        # Up to +-2 steps of the grid: frequency steps of resolution/20,
        # DM steps of half the plan step.
        f = 1 / TRUE_P + rng.uniform(-2, 2) * resolution / 20
        starts.append((1 / f, 0.0, TRUE_DM + rng.uniform(-2, 2) * step / 2))
    grid, rcs = fold.refine_grid(fb, N, starts, resolution, step, 0.0, 150.0, 128)
    for exact in (True, False):
        out, J, ev = fold.refine_gradient(fb, N, starts, 128, 64, exact=exact)
        out = mid_epoch(out, T)
        for i in range(len(starts)):
            # Both land on the injected signal; the gradient result is no
            # farther from the truth than the grid's (whose steps quantise it).
            assert abs(out[i]["dm"] - TRUE_DM) <= \
                max(abs(grid[i]["dm"] - TRUE_DM), step / 4) + 0.02, (exact, out[i], grid[i])
            assert abs(out[i]["period_s"] - TRUE_P) <= \
                max(abs(grid[i]["period_s"] - TRUE_P), TRUE_P ** 2 * resolution / 40) + 1e-9, \
                (exact, out[i], grid[i])
            assert ev[i] <= 40


@pytest.mark.gpu
def test_device_synth_statistics_and_determinism(gpu):
    from pulsarsr_gb300 import synth
    a = synth.device(16, 32, 1 << 16, 64e-6, 1500.0, -10.0, seed=9, noise_mean=3.0,
                     noise_sigma=2.0)
    b = synth.device(16, 32, 1 << 16, 64e-6, 1500.0, -10.0, seed=9, noise_mean=3.0,
                     noise_sigma=2.0)
    c = synth.device(16, 8, 1 << 16, 64e-6, 1500.0, -10.0, seed=9, noise_mean=100.0,
                     noise_sigma=10.0)
    x, y, z = a.data, b.data, c.data
    assert x.tobytes() == y.tobytes()
    assert abs(x.mean() - 3.0) < 0.02 and abs(x.std() - 2.0) < 0.02
    assert abs(z.mean() - 100.0) < 0.2 and z.min() >= 0 and z.max() <= 255
    assert np.all(z == np.rint(z))
    # neighbouring samples and channels are uncorrelated
    r = np.corrcoef(x[:, :-1].ravel(), x[:, 1:].ravel())[0, 1]
    assert abs(r) < 0.01


@pytest.mark.gpu
def test_refinement_on_device_synthesised_pulsar(gpu):
    """A 256-channel 2^20-sample f32 observation made on the device with one
    pulsar (P 8.7 ms, DM 213.4); the gradient and grid refinements from offset
    starts both recover it."""
    from pulsarsr_gb300 import dedisperse, fold, synth
    P, PD, DM = 0.0087341, 0.0, 213.4
    fb = synth.device(256, 32, 1 << 20, 64e-6, 1500.0, -400.0 / 256, seed=11,
                      pulsars=[synth.Pulsar(P, DM, 0.04, 0.08, phase=0.3, pdot=PD)])
    freqs = fb.header.frequencies()
    n = fb.nsamples - int(dedisperse.delays(freqs, 64e-6, 400.0).max()) - 4
    T = n * 64e-6
    resolution = 1.0 / T
    step = dedisperse.dm_step(freqs, 64e-6)
    rng = np.random.default_rng(3)
    starts = [(1 / (1 / P + rng.uniform(-2, 2) * resolution / 20), 0.0,
               DM + rng.uniform(-2, 2) * step / 2) for _ in range(16)]
    out, J, ev = fold.refine_gradient(fb, n, starts, 128, 64)
    out = mid_epoch(out, T)
    grid, _ = fold.refine_grid(fb, n, starts, resolution, step, 0.0, 400.0, 128)
    dp_grad = np.abs(out["period_s"] - P)
    dp_grid = np.abs(grid["period_s"] - P)
    dd_grad = np.abs(out["dm"] - DM)
    dd_grid = np.abs(grid["dm"] - DM)
    assert np.median(dp_grad) <= np.median(dp_grid) + P * P * resolution / 40
    assert np.median(dd_grad) <= np.median(dd_grid) + step / 8
    assert np.all(dp_grad < P * P * resolution / 4) and np.all(dd_grad < step)


def cube_objective_np(x, freqs, tsamp, n, P, pdot, dm, B):
    """J of the cube at its reference point (every shift zero): every
    channel's samples [0, n) folded with cloud-in-cell weights at its own
    dispersed phase, summed over channels, J = sum_b (p_b - mean)^2 / (n v),
    v = sum of the channels' variances (f64 per sample)."""
    nu = 1.0 / P
    nudot = -pdot * nu * nu
    fmax = freqs.max()
    kc = 4148.808 * (1.0 / freqs ** 2 - 1.0 / fmax ** 2)
    t = np.arange(n) * tsamp
    prof = np.zeros(B)
    v = 0.0
    for c in range(x.shape[0]):
        xc = x[c, :n].astype(np.float64)
        td = t - kc[c] * dm
        ph = nu * td + 0.5 * nudot * td * td
        u = (ph - np.floor(ph)) * B
        b0 = np.floor(u).astype(np.int64)
        w = u - b0
        b0 %= B
        prof += np.bincount(b0, (1 - w) * xc, B) + np.bincount((b0 + 1) % B, w * xc, B)
        v += xc.var()
    return float(((prof - prof.mean()) ** 2).sum() / (n * v))


@pytest.mark.gpu
@pytest.mark.parametrize("nbits,P,pdot", [(8, 0.0237, 0.0), (8, 0.0041, 2e-9),
                                          (32, 0.0237, -1e-9), (32, 0.0041, 0.0),
                                          (8, 1.3, 0.0), (8, 0.2, 5e-9), (16, 0.05, 0.0)])
def test_cube_objective_matches_numpy_fold(gpu, nbits, P, pdot):
    """The folded cube (one CTA per channel and subint, 32-sample runs,
    fixed-point phases) against a plain f64 fold: J at the cube's reference
    point, which refine_gradient returns after one evaluation.  Slow (< 1 bin
    per sample) and fast pulsars, 8-bit and f32 data, n not a multiple of the
    run length or the subint count."""
    from pulsarsr_gb300 import fold, synth
    DM = 57.3
    fb = synth.device(48, nbits, 1 << 17, 64e-6, 1500.0, -400.0 / 48, seed=21,
                      noise_mean={8: 100.0, 16: 3000.0}.get(nbits, 0.0),
                      noise_sigma={8: 12.0, 16: 300.0}.get(nbits, 1.0),
                      pulsars=[synth.Pulsar(P, DM, 0.05, 0.3, phase=0.2, pdot=pdot)])
    x = fb.data
    n = (1 << 17) - 3001
    _, J, ev = fold.refine_gradient(fb, n, [(P, pdot, DM)], 128, 64, max_evals=1)
    assert ev[0] == 1
    Jn = cube_objective_np(x, fb.header.frequencies(), 64e-6, n, P, pdot, DM, 128)
    assert np.isclose(J[0], Jn, rtol=2e-4), (J[0], Jn)
