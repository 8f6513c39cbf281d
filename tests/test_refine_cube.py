"""The folded-cube objective of the default gradient refinement and its
hand-written adjoint (psr_refine_cube_objective), in the three fold regimes
of the cube kernels (du = bins per sample < 1/31: 32-sample runs; 1/31 <= du
< 1: bin-owner gather; du >= 1: private bin columns).

The FP64 model below restates the cube objective in numpy: every channel's
subint rows folded with cloud-in-cell weights at the reference, row means
removed, rows taken to the Fourier domain, each row's harmonics shifted by
its phase change at the subint centre, J by Parseval, and the adjoint
  dJ/dd_cs = sum_k Re(A_k R_cs[k] e^(-2 pi i k d_cs/B) (-2 pi i k/B)),
  A_k = 2 w_k conj(P_k) / (B n v).
On the CPU the model's adjoint is checked against central differences of the
model itself; on the GPU the device objective and adjoint are checked
against the model and against central differences of the device objective.
Gradients are compared as directional changes g_i h_i over steps h_i that
move the last sample by a fixed fraction of a bin, so that P, Pdot and DM
weigh alike; tolerances relative to the largest of them."""
import numpy as np
import pytest

K_DM = 4148.808
B, S = 128, 64


def chan_consts(freqs):
    return K_DM * (1.0 / freqs ** 2 - 1.0 / freqs.max() ** 2)


def cube_f64(x, freqs, tsamp, n, ref):
    """Rows R[c, s, k-1] = sum_b C[c, s, b] e^(-2 pi i k b / B), k = 1..B/2, of
    the cube folded at ref = (P, Pdot, DM), and v = sum of channel variances."""
    P, Pd, dm = ref
    nu, nud = 1.0 / P, -Pd / P ** 2
    kc = chan_consts(freqs)
    nch = x.shape[0]
    C = np.zeros((nch, S, B))
    t = np.arange(n) * tsamp
    v = 0.0
    for c in range(nch):
        xc = x[c, :n].astype(np.float64)
        td = t - kc[c] * dm
        ph = nu * td + 0.5 * nud * td * td
        u = (ph - np.floor(ph)) * B
        b0 = np.floor(u).astype(np.int64)
        w = u - b0
        b0 %= B
        for s in range(S):
            t0, t1 = n * s // S, n * (s + 1) // S
            sl = slice(t0, t1)
            row = np.bincount(b0[sl], (1 - w[sl]) * xc[sl], B) + \
                np.bincount((b0[sl] + 1) % B, w[sl] * xc[sl], B)
            C[c, s] = row - row.mean()
        v += xc.var()
    R = np.fft.fft(C, axis=-1)[..., 1:B // 2 + 1]
    return R, v


def objective_f64(R, v, freqs, tsamp, n, ref, theta):
    """J and dJ/d(P, Pdot, DM) of the cube model at theta."""
    P0, Pd0, dm0 = ref
    P, Pd, dm = theta
    nu0, nud0 = 1.0 / P0, -Pd0 / P0 ** 2
    nu, nud = 1.0 / P, -Pd / P ** 2
    kc = chan_consts(freqs)[:, None]
    Ts = (np.arange(S) + 0.5) * (n * tsamp / S)
    tdr = Ts[None, :] - kc * dm0
    tdq = Ts[None, :] - kc * dm
    d = B * ((nu * tdq + 0.5 * nud * tdq ** 2) - (nu0 * tdr + 0.5 * nud0 * tdr ** 2))
    k = np.arange(1, B // 2 + 1)
    E = np.exp(-2j * np.pi * k[None, None, :] * d[:, :, None] / B)
    Pk = (R * E).sum(axis=(0, 1))
    wk = np.where(k < B // 2, 2.0, 1.0)
    norm = B * n * v
    J = float((wk * np.abs(Pk) ** 2).sum() / norm)
    A = 2 * wk * np.conj(Pk) / norm
    gd = np.real((A[None, None, :] * R * E * (-2j * np.pi * k[None, None, :] / B)).sum(axis=2))
    g_nu = float((gd * B * tdq).sum())
    g_nud = float((gd * B * 0.5 * tdq ** 2).sum())
    g_dm = float((gd * (-B * (nu + nud * tdq) * kc)).sum())
    # (nu, nudot) = (1/P, -Pdot/P^2)
    g_P = g_nu * (-1.0 / P ** 2) + g_nud * (2.0 * Pd / P ** 3)
    g_Pd = g_nud * (-1.0 / P ** 2)
    return J, np.array([g_P, g_Pd, g_dm])


def steps(freqs, tsamp, n, theta, bins_moved):
    """Steps in P, Pdot and DM that move the last sample (or the lowest
    channel) by `bins_moved` phase bins."""
    P = theta[0]
    T = n * tsamp
    hP = bins_moved * P * P / (B * T)
    hPd = 2.0 * bins_moved * P * P / (B * T * T)
    hD = bins_moved * P / (B * chan_consts(freqs).max())
    return np.array([hP, hPd, hD])


def central(f, theta, h):
    out = np.zeros(3)
    for i in range(3):
        e = np.zeros(3)
        e[i] = h[i]
        out[i] = (f(theta + e) - f(theta - e)) / 2.0
    return out


# (nbits, P, Pdot): du = 128 * 64e-6 / P = 0.0063 (runs), 0.35 (bin-owner
# gather), 2.0 (private columns)
REGIMES = [(8, 1.3, 0.0), (32, 0.0237, -1e-9), (8, 0.0041, 2e-9)]


def synthetic(nbits, P, Pd, nch=24, ns=1 << 15, seed=3):
    """A small host filterbank with one pulsar (for the CPU check)."""
    rng = np.random.default_rng(seed)
    tsamp = 64e-6
    freqs = 1500.0 - np.arange(nch) * 400.0 / nch
    kc = chan_consts(freqs)
    t = np.arange(ns) * tsamp
    x = rng.standard_normal((nch, ns))
    for c in range(nch):
        td = t - kc[c] * 57.3
        ph = np.mod(td / P - 0.5 * Pd * td * td / P ** 2 - 0.2, 1.0)
        dist = np.minimum(ph, 1 - ph)
        x[c] += 0.5 * np.exp(-0.5 * (dist / (0.05 / 2.355)) ** 2)
    return x, freqs, tsamp


@pytest.mark.parametrize("nbits,P,Pd", REGIMES)
def test_cube_model_adjoint_matches_finite_differences(nbits, P, Pd):
    x, freqs, tsamp = synthetic(nbits, P, Pd)
    n = x.shape[1] - 2000
    ref = (P, Pd, 57.3)
    R, v = cube_f64(x, freqs, tsamp, n, ref)
    theta = np.array(ref) + steps(freqs, tsamp, n, np.array(ref), 0.3)
    J, g = objective_f64(R, v, freqs, tsamp, n, ref, theta)
    h = steps(freqs, tsamp, n, theta, 1e-3)
    fd = central(lambda th: objective_f64(R, v, freqs, tsamp, n, ref, th)[0], theta, h)
    scale = np.abs(g * h).max()
    assert scale > 0
    assert np.allclose(g * h, fd, rtol=0, atol=1e-6 * scale), (g * h, fd)


@pytest.mark.gpu
@pytest.mark.parametrize("nbits,P,Pd", REGIMES)
def test_device_cube_objective_and_adjoint(gpu, nbits, P, Pd):
    """Device J and adjoint against the FP64 model, and against central
    differences of the device objective itself.  The device folds f32 cube
    cells and rotates harmonics in f32: measured on a GB300, J within 3e-7
    of the model and the gradient's directional changes within 9e-5 of the
    largest; the bounds below leave a margin of about 10x.  The secant of
    the device J over 0.01-bin steps magnifies its f32 rounding (2e-2)."""
    from pulsarsr_gb300 import fold, synth
    DM = 57.3
    fb = synth.device(48, nbits, 1 << 17, 64e-6, 1500.0, -400.0 / 48, seed=21,
                      noise_mean={8: 100.0, 16: 3000.0}.get(nbits, 0.0),
                      noise_sigma={8: 12.0, 16: 300.0}.get(nbits, 1.0),
                      pulsars=[synth.Pulsar(P, DM, 0.05, 0.3, phase=0.2, pdot=Pd)])
    x = fb.data
    freqs = fb.header.frequencies()
    n = (1 << 17) - 3001
    ref = (P, Pd, DM)
    R, v = cube_f64(x, freqs, 64e-6, n, ref)
    base = np.array(ref)
    pts = [base, base + steps(freqs, 64e-6, n, base, 0.3),
           base + steps(freqs, 64e-6, n, base, -0.6) * np.array([1.0, -1.0, 0.5])]
    J, g = fold.refine_cube_objective(fb, n, ref, pts, B, S)
    for i, th in enumerate(pts):
        Jm, gm = objective_f64(R, v, freqs, 64e-6, n, ref, th)
        assert np.isclose(J[i], Jm, rtol=3e-6), (i, J[i], Jm)
        h = steps(freqs, 64e-6, n, th, 1.0)
        scale = np.abs(gm * h).max()
        assert np.allclose(g[i] * h, gm * h, rtol=0, atol=1e-3 * scale), (i, g[i] * h, gm * h)
    th = pts[1]
    h = steps(freqs, 64e-6, n, th, 1e-2)
    probe = []
    for j in range(3):
        e = np.zeros(3)
        e[j] = h[j]
        probe += [th + e, th - e]
    Jp, _ = fold.refine_cube_objective(fb, n, ref, probe, B, S)
    fd = (Jp[0::2] - Jp[1::2]) / 2.0
    scale = np.abs(g[1] * h).max()
    assert np.allclose(g[1] * h, fd, rtol=0, atol=2e-2 * scale), (g[1] * h, fd)
