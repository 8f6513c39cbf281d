"""Benchmark of the PulsarSr search hot path on GB300.

Workload (default): the GBT L-band-shaped observation -- 96 x 1 MHz
channels, 4-bit, 72 us, 531000 samples, seeded synthetic data with a
4.6214 ms pulsar at DM 62.4, a 28.76 Hz zero-DM tone and 5 bursts -- searched
over the default DM plan 0-500 (2000 trials, step 0.25006), RFI masking on,
15-2000 Hz, threshold 8, 32 candidates per trial.

A step is one whole search of the observation: unpack -> RFI mask -> for
every trial DM dedisperse -> real FFT + power -> normalise -> harmonic sums
-> per-trial candidate list.  metric: DM-trial*samples per second
(trials x discovery samples / step time).

  value : device-resident (packed payload already in HBM), CUDA events on the
          session stream, L2 flushed (512 MB memset) before every step.
  e2e   : through the public API with host buffers: payload H2D from pinned
          memory, run, sync, candidate lists D2H, host wall clock.
  --impl reference : the CPU restatement of the reference's path (the Rust
          reference cannot be built here) timed on the host cores.
"""
from __future__ import annotations

import argparse
import ctypes as C
import glob
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "search DM-trial*samples/s (GBT-shaped 2000-trial search)"
UNIT = "DM-trial*samples/s"


# ------------------------------------------------------------ cudart
def cudart():
    for p in ["libcudart.so"] + sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*")):
        try:
            return C.CDLL(p)
        except OSError:
            continue
    raise RuntimeError("libcudart not found")


class Events:
    def __init__(self, rt):
        self.rt = rt

    def new(self):
        e = C.c_void_p()
        assert self.rt.cudaEventCreate(C.byref(e)) == 0
        return e

    def record(self, e, stream):
        assert self.rt.cudaEventRecord(e, C.c_void_p(stream)) == 0

    def ms(self, a, b):
        assert self.rt.cudaEventSynchronize(b) == 0
        v = C.c_float()
        assert self.rt.cudaEventElapsedTime(C.byref(v), a, b) == 0
        return v.value


# ------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.rows = []
        self.proc = None
        self.idx = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm = [float(r[0]) for r in self.rows if len(r) >= 8 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 8 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 8 for i in range(4)
                          if r[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(sm)}


# ------------------------------------------------------------ workload
def workload(name: str, planner=None):
    """The observation, its payload, DM plan and discovery length.  planner
    supplies dm_step/plan/delays: libpsr by default, the oracle for the
    reference arm (so that arm never maps libpsr)."""
    from pulsarsr_gb300 import synth
    if planner is None:
        from pulsarsr_gb300 import dedisperse as planner
    dedisperse = planner
    obs = synth.config_c2(2) if name == "c2" else synth.config_c1(1)
    raw = obs.to_bytes()
    freqs = obs.frequencies()
    step = dedisperse.dm_step(freqs, obs.tsamp)
    dm_max = 500.0 if name == "c2" else 120.0
    trials = dedisperse.plan(0.0, dm_max, step if name == "c2" else 2.0)
    md = int(dedisperse.delays(freqs, obs.tsamp, dm_max).max())
    length = obs.nsamples - md
    discovery = (length - md) // 2
    return obs, raw, trials, discovery


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def stage_bytes(stage, obs, trials, discovery, N, chunk=256, masked_fraction=0.0):
    """Algorithmic HBM bytes of one whole search, per stage.

    Per unit: dedispersion reads the packed observation once per block of
    `chunk` trials and writes 4 bytes per output sample; the rFFT reads the
    series (4*discovery, the zero padding is not read) and writes 4*(N/2+1)
    power bins; normalisation + harmonic sums read the 4*(N/2+1) bins; RFI
    reads the samples once and writes the masked ones; unpack reads the
    payload and writes one byte per sample.  Intermediates (the FFT work
    buffer, partial sums) are not algorithmic bytes.
    """
    nt, nch, ns = len(trials), obs.nchans, obs.nsamples
    payload = (ns * nch * obs.nbits) // 8
    bins = N // 2 + 1
    if stage == "dedisperse":
        return payload * -(-nt // chunk) + 4 * nt * discovery
    if stage == "fft":
        return nt * (4 * discovery + 4 * bins)
    if stage == "spectrum":
        return nt * 4 * bins
    if stage == "rfi":
        return nch * ns + int(nch * ns * masked_fraction)
    if stage == "unpack":
        return payload + ns * nch
    return 0


def measured_traffic(stage):
    """ncu DRAM bytes per trial for a stage's kernels (profiles/traffic.json)."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p)).get(stage)
    if not d:
        return None
    return d["dram_bytes_per_launch"] / d["trials_per_launch"]


def measured_instructions(stage):
    """ncu warp instructions per trial for a stage's kernels (profiles/traffic.json)."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p)).get(stage)
    if not d or "warp_instructions_per_launch" not in d:
        return None
    return d["warp_instructions_per_launch"] / d["trials_per_launch"]


def max_over_ranks(x: float, dist) -> float:
    """The slowest rank's value (all ranks get it); x itself without a group."""
    if not dist:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: float, ms: float, world: int) -> float:
    """Whole-job rate of `world` replicas that each process units_per_rank
    units, timed by the slowest rank (weak scaling)."""
    return world * units_per_rank / (ms / 1e3)


def run_ours(args):
    from pulsarsr_gb300 import fbank, search, session
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # plumbing only: barrier + max over ranks
        dist.init_process_group("gloo")
    local = int(os.environ.get("LOCAL_RANK", "0"))
    rt = cudart()
    rt.cudaSetDevice(C.c_int(local))
    obs, raw, trials, discovery = workload(args.config)
    if args.trials:
        trials = trials[:args.trials]
    hdr = fbank.parse_header(raw)
    payload = np.frombuffer(raw, dtype=np.uint8)[hdr.data_offset:].copy()
    # pinned host payload for the e2e leg
    assert rt.cudaHostRegister(C.c_void_p(payload.ctypes.data), C.c_size_t(payload.nbytes),
                               C.c_uint(0)) == 0
    cfg = search.Config(min_hz=15.0, max_hz=2000.0, threshold=8.0, max_candidates=32)
    block = max(int(0.1 / obs.tsamp), 32)
    s = session.SearchSession(hdr, obs.nsamples, trials, discovery, cfg, block, 8.0)
    s.load(payload)
    flush = C.c_void_p()
    FLUSH = 512 << 20
    assert rt.cudaMalloc(C.byref(flush), C.c_size_t(FLUSH)) == 0
    ev = Events(rt)
    stream = s.stream
    for _ in range(args.warmup):
        s.run()
        s.sync()
    # ---- device-resident timing
    if dist:
        dist.barrier()
    rt.cudaDeviceSynchronize()
    clocks = ClockSampler(local)
    clocks.start()
    times = []
    for _ in range(args.steps):
        rt.cudaMemsetAsync(flush, C.c_int(0), C.c_size_t(FLUSH), C.c_void_p(stream))
        a, b = ev.new(), ev.new()
        ev.record(a, stream)
        s.run()
        ev.record(b, stream)
        s.sync()
        times.append(ev.ms(a, b))
    rt.cudaDeviceSynchronize()
    clk = clocks.stop()
    ms = max_over_ranks(statistics.mean(times), dist)
    units = len(trials) * discovery
    value = replica_throughput(units, ms, world)
    counts, cands = s.candidates()
    # ---- end to end through the public API with host buffers
    e2e = []
    for _ in range(max(args.steps // 2, 2)):
        rt.cudaDeviceSynchronize()
        t0 = time.perf_counter()
        s.load(payload)
        s.run()
        s.sync()
        c2, k2 = s.candidates()
        e2e.append(time.perf_counter() - t0)
    e2e_s = statistics.mean(e2e)
    d2h = counts.nbytes + len(trials) * 32 * 40
    # ---- per-stage profile (separate runs; events per stage launch)
    s.set_profiling(True)
    s.stage_times(reset=True)
    for _ in range(2):
        rt.cudaMemsetAsync(flush, C.c_int(0), C.c_size_t(FLUSH), C.c_void_p(stream))
        s.run()
        s.sync()
    st = s.stage_times()
    # The same with the stages serialised: each stage's kernels alone.
    s.set_profiling(2)
    s.stage_times(reset=True)
    for _ in range(2):
        rt.cudaMemsetAsync(flush, C.c_int(0), C.c_size_t(FLUSH), C.c_void_p(stream))
        s.run()
        s.sync()
    st_iso = s.stage_times()
    s.set_profiling(False)
    N = 2 * (1 << (discovery - 1).bit_length())
    # The dominant kernels are the rFFT stage's (k_fft_pass1 + k_fft_pass2, one
    # event pair per inner chunk of trials).
    peak, src = peaks()
    mfrac = s.mask()["masked_fraction"]
    stages = {}
    for k in ("unpack", "rfi", "dedisperse", "fft", "spectrum"):
        tot_ms, nl = st[k]
        if nl == 0:
            continue
        ms_search = tot_ms / 2
        nbytes = stage_bytes(k, obs, trials, discovery, N, masked_fraction=mfrac)
        iso = st_iso[k][0] / 2
        stages[k] = {"ms_per_search": round(ms_search, 4), "event_pairs_per_search": nl // 2,
                     "ms_per_event_pair": round(tot_ms / nl, 5),
                     "algorithmic_gb": round(nbytes / 1e9, 4),
                     "gbs": round(nbytes / (ms_search / 1e3) / 1e9, 1),
                     "ms_per_search_serialised": round(iso, 4),
                     "gbs_serialised": round(nbytes / (iso / 1e3) / 1e9, 1) if iso else None}
    # Dedispersion against its ALU bound: sample-adds (nch per DM-trial*sample)
    # packed 4 per 32-bit add for <= 4-bit samples (byte lanes), 2 otherwise
    # (16-bit lanes), against 128 32-bit integer adds per clock per SM at the
    # SM clock sampled during the timed steps.
    if "dedisperse" in stages:
        nsm = C.c_int(0)
        rt.cudaDeviceGetAttribute(C.byref(nsm), C.c_int(16), C.c_int(local))  # SM count
        mhz = (clk.get("sm_mhz") or 2070.0)
        lanes = 4 if obs.nbits <= 4 else 2
        word_adds = obs.nchans * len(trials) * discovery / lanes
        dd_s = stages["dedisperse"]["ms_per_search"] / 1e3
        dd_iso = stages["dedisperse"]["ms_per_search_serialised"] / 1e3
        peak_adds = nsm.value * 128 * mhz * 1e6
        stages["dedisperse"]["issue_frac"] = round(word_adds / dd_s / peak_adds, 4)
        stages["dedisperse"]["issue_frac_serialised"] = round(word_adds / dd_iso / peak_adds, 4)
        stages["dedisperse"]["issue_basis"] = (
            f"{obs.nchans} x {len(trials)} x {discovery} sample-adds / {lanes} per 32-bit add "
            f"vs {nsm.value} SMs x 128 int32 adds/clk x {mhz:.0f} MHz")
    D = st["dedisperse"][1] // 2
    F = st["fft"][1] // 2
    fft_kernels = 2 if N // 2 > 4096 else 1
    # unpack + 9 RFI kernels (8-bit storage: totals, mean/variance, block sums,
    # median histograms + pick, channel and block decisions, block means,
    # fill); per outer chunk dedispersion + part reduction + harmonic items +
    # selection; per inner chunk the FFT pass(es) and the scales/gates kernel
    launches = 1 + 9 + D * 4 + F * (fft_kernels + 1)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    # Per launch of the dominant kernels: algorithmic bytes of the trials one
    # launch processes / the launch's average CUDA-event duration.
    fft_ms, fft_pairs = st["fft"]
    launches_per_search = fft_pairs / 2
    trials_per_launch = len(trials) / launches_per_search
    ms_per_launch = fft_ms / fft_pairs
    alg_per_launch = stage_bytes("fft", obs, trials, discovery, N) / launches_per_search
    achieved = alg_per_launch / (ms_per_launch / 1e3) / 1e9
    # ncu figures per trial were captured on the GBT-shaped case (the rFFT of
    # 2^20 points); other shapes report none.
    gbt = args.config == "c2"
    per_trial = measured_traffic("fft") if gbt else None
    traffic = per_trial * trials_per_launch if per_trial else None
    # The rFFT against its issue bound: warp instructions per trial (ncu, the
    # same kernels on the 64-trial case) over the serialised stage time and
    # 4 warp instructions per clock per SM at the sampled SM clock.
    ipt = measured_instructions("fft") if gbt else None
    fft_iso = stages.get("fft", {}).get("ms_per_search_serialised")
    issue = None
    if ipt and fft_iso:
        nsm_f = C.c_int(0)
        rt.cudaDeviceGetAttribute(C.byref(nsm_f), C.c_int(16), C.c_int(local))
        mhz_f = clk.get("sm_mhz") or 2070.0
        issue = {"warp_instructions_per_trial": round(ipt),
                 "frac": round(ipt * len(trials) / (fft_iso / 1e3)
                               / (nsm_f.value * 4 * mhz_f * 1e6), 4),
                 "basis": "warp instructions per trial (profiles/traffic.json) x trials / "
                          "serialised FFT stage time, vs 4 warp instructions per clock per "
                          f"SM x {nsm_f.value} SMs x {mhz_f:.0f} MHz"}
    cpu = cpu_baseline(obs, raw, trials, discovery, args) if not args.no_cpu else None
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/f32",
        "data": "synthetic (seeded numpy generator, GBT L-band tutorial shape)",
        "config": search_config(args, obs, trials, discovery, world),
        "e2e": {"value": round(world * units / e2e_s, 1), "unit": UNIT,
                "h2d_bytes_per_step": int(payload.nbytes), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "k_fft_pass1 + k_fft_pass2 (rFFT + power)",
                     "trials_per_launch": round(trials_per_launch, 3),
                     "algorithmic_bytes_per_launch": int(alg_per_launch),
                     "ms_per_launch": round(ms_per_launch, 5),
                     "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": int(traffic) if traffic else None,
                     "traffic_source": "profiles/traffic.json (ncu, cold L2), per trial x "
                                       "trials_per_launch",
                     "peak_source": src, "issue": issue},
        "stages": stages,
        "clocks": clk,
        "candidates": int(counts.sum()),
    }
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def cpu_baseline(obs, raw, trials, discovery, args, sample_trials=None):
    """The oracle (CPU restatement of the reference path) on a bounded sample:
    decode + RFI once, then `sample_trials` trial DMs spread over the plan on
    all host threads; the full-plan time is extrapolated per trial (exact
    when the sample is the whole plan)."""
    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    # about 10-30 core-seconds of trial work on a 16-core host (320 of the
    # GBT-shaped plan's 2000 trials), never more than the plan
    nsample = min(sample_trials or max(2 * threads, 320), len(trials))
    t0 = time.perf_counter()
    h, d = O.decode(raw)
    block = max(int(0.1 / obs.tsamp), 32)
    md, _ = O.rfi_mask(d, block, 8.0)
    t_pre = time.perf_counter() - t0
    pick = np.linspace(0, len(trials) - 1, nsample).astype(int)
    t1 = time.perf_counter()
    O.search_trials(md, obs.frequencies(), obs.tsamp, trials[pick], discovery, threads=threads,
                    min_hz=15.0, max_hz=2000.0, threshold=8.0, max_candidates=32)
    t_tr = time.perf_counter() - t1
    full = t_pre + t_tr * len(trials) / nsample
    value = len(trials) * discovery / full
    if nsample == len(trials):
        sample = (f"whole search: decode+RFI ({t_pre:.2f}s) + all {len(trials)} trials "
                  f"({t_tr:.2f}s on {threads} threads)")
    else:
        sample = (f"decode+RFI once ({t_pre:.2f}s) + {nsample} of {len(trials)} trials "
                  f"({t_tr:.2f}s on {threads} threads), extrapolated to the full plan "
                  f"({full:.1f}s)")
    return {"value": round(value, 1), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": sample}


def search_config(args, obs, trials, discovery, world):
    """The `config` object of the search lines (both arms)."""
    N = 2 * (1 << (discovery - 1).bit_length())
    return {"workload": f"{'GBT-shaped' if args.config == 'c2' else 'config-1'} search: "
                        f"{obs.nchans} ch x {obs.nbits}-bit x {obs.nsamples} samples, "
                        f"tsamp {obs.tsamp * 1e6:.0f} us, {len(trials)} DM trials, "
                        f"discovery {discovery}, rFFT {N}, RFI on",
            "trials": len(trials), "discovery_samples": discovery,
            "l2": "flushed (512 MB memset) before every timed step",
            "parallelism": f"replicas x{world}"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    obs, raw, trials, discovery = workload(args.config, planner=O)
    vals = []
    info = None
    # Warm-up steps search a 320-trial sample; every timed step is a whole
    # search of the full plan (about 6 s on 16 host cores for the GBT shape).
    for i in range(args.warmup + args.steps):
        timed = i >= args.warmup
        info = cpu_baseline(obs, raw, trials, discovery, args,
                            sample_trials=len(trials) if timed else None)
        if timed:
            vals.append(info["value"])
    v = statistics.mean(vals)
    info = dict(info)
    info["value"] = round(v, 1)
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 1), "unit": UNIT,
            "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32/f64 (CPU)",
            "data": "synthetic (seeded numpy generator, GBT L-band tutorial shape)",
            "config": search_config(args, obs, trials, discovery,
                                    int(os.environ.get("WORLD_SIZE", "1"))),
            "cpu_baseline": info,
            "e2e": {"value": round(v, 1), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "PulsarSr is Rust; cargo/rustc are absent, so the timed CPU path is the "
                    "C++ restatement of its search path (oracle/), validated against the "
                    "reference's saved reports"}
    print(json.dumps(line))


# ------------------------------------------------------------ refinement
def refine_workload(seed=4):
    """1024 ch f32, 2^23 samples at 64 us, 1100-1500 MHz, generated on the
    device: N(0,1) noise plus 16 seeded pulsars (P 5-500 ms log-uniform, DM
    10-300, duty 3-5%); 16 starting points per pulsar offset uniformly by up
    to +-2 grid steps in frequency (resolution / 20) and DM (half the plan
    step)."""
    from pulsarsr_gb300 import dedisperse, synth
    rng = np.random.default_rng(seed)
    nch, ns, tsamp, fch1, foff = 1024, 1 << 23, 64e-6, 1500.0, -400.0 / 1024
    pulsars = []
    for _ in range(16):
        P = float(np.exp(rng.uniform(np.log(0.005), np.log(0.5))))
        pulsars.append(synth.Pulsar(P, float(rng.uniform(10, 300)), float(rng.uniform(0.03, 0.05)),
                                    float(rng.uniform(0.002, 0.005)),
                                    phase=float(rng.uniform(0, 1))))
    fb = synth.device(nch, 32, ns, tsamp, fch1, foff, seed=seed, pulsars=pulsars)
    freqs = fb.header.frequencies()
    n = ns - int(dedisperse.delays(freqs, tsamp, 400.0).max()) - 4
    resolution = 1.0 / (n * tsamp)
    step = dedisperse.dm_step(freqs, tsamp)
    starts, truth = [], []
    for p in pulsars:
        for _ in range(16):
            f = 1 / p.period_s + rng.uniform(-2, 2) * resolution / 20
            starts.append((1 / f, 0.0, p.dm + rng.uniform(-2, 2) * step / 2))
            truth.append((p.period_s, 0.0, p.dm))
    return fb, n, starts, np.array(truth), resolution, step, tsamp


def run_refine(args):
    from pulsarsr_gb300 import fold
    rt = cudart()
    t0 = time.perf_counter()
    fb, n, starts, truth, resolution, step, tsamp = refine_workload()
    rt.cudaDeviceSynchronize()
    t_synth = time.perf_counter() - t0
    T = n * tsamp
    # warm-up on a few candidates (module loads, allocations)
    # The gradient's DM is kept inside the window the grid searches (10 half steps).
    window = 10 * step / 2
    fold.refine_gradient(fb, n, starts[:16], dm_window=window)
    fold.refine_grid(fb, n, starts[:2], resolution, step, 0.0, 400.0, 128)
    rt.cudaDeviceSynchronize()
    t0 = time.perf_counter()
    g, J, ev = fold.refine_gradient(fb, n, starts, dm_window=window)
    rt.cudaDeviceSynchronize()
    t_grad = time.perf_counter() - t0
    t0 = time.perf_counter()
    q, rcs = fold.refine_grid(fb, n, starts, resolution, step, 0.0, 400.0, 128)
    rt.cudaDeviceSynchronize()
    t_grid = time.perf_counter() - t0
    # A finer grid, refined to the 1e-9 s / 0.01 tolerance: two more levels
    # of the same grid method around the coarse result, frequency spacing
    # resolution/400 then resolution/8000 (P spacing P^2/(8000 T): 6e-10 s at
    # P = 50 ms), DM half steps 0.01 then 0.001.
    t0 = time.perf_counter()
    q2, _ = fold.refine_grid(fb, n, [tuple(x) for x in q], resolution / 20, 0.02, 0.0, 400.0, 128)
    q3, _ = fold.refine_grid(fb, n, [tuple(x) for x in q2], resolution / 400, 0.002, 0.0, 400.0,
                             128)
    rt.cudaDeviceSynchronize()
    t_fine = time.perf_counter() - t0
    pm_grad = g["period_s"] + g["pdot"] * T / 2  # period at mid-span
    dp_grad = np.abs(pm_grad - truth[:, 0])
    dp_grid = np.abs(q["period_s"] - truth[:, 0])
    dd_grad = np.abs(g["dm"] - truth[:, 2])
    dd_grid = np.abs(q["dm"] - truth[:, 2])
    gg_p = np.abs(pm_grad - q["period_s"])
    gg_d = np.abs(g["dm"] - q["dm"])
    gf_p = np.abs(pm_grad - q3["period_s"])
    gf_d = np.abs(g["dm"] - q3["dm"])
    dp_fine = np.abs(q3["period_s"] - truth[:, 0])
    dd_fine = np.abs(q3["dm"] - truth[:, 2])
    # the coarse grid's own quantum: frequency steps resolution/20, DM half steps
    p_quant = np.median(truth[:, 0] ** 2 * resolution / 20)
    ncand = len(starts)
    line = {
        "metric": "refine s/candidate (gradient vs grid, 256 candidates)",
        "value": round(t_grad / ncand, 6), "unit": "s/candidate", "n_gpus": 1,
        "higher_is_better": False, "dtype": "f32 data, f64 phases",
        "data": "synthetic, generated on the device (seed 4)",
        "config": {"workload": "1024 ch f32 x 2^23 samples, 64 us, 1100-1500 MHz, 16 pulsars, "
                               "256 starts offset <= 2 grid steps; 128 bins x 64 subints",
                   "n": int(n), "candidates": ncand},
        "grid_s_per_candidate": round(t_grid / ncand, 6),
        "speedup_vs_grid": round(t_grid / t_grad, 2),
        "synth_seconds": round(t_synth, 3),
        "evaluations_median": int(np.median(ev)),
        "period_error_s": {"gradient_median": float(np.median(dp_grad)),
                           "gradient_p90": float(np.percentile(dp_grad, 90)),
                           "grid_median": float(np.median(dp_grid)),
                           "grid_p90": float(np.percentile(dp_grid, 90))},
        "dm_error": {"gradient_median": float(np.median(dd_grad)),
                     "gradient_p90": float(np.percentile(dd_grad, 90)),
                     "grid_median": float(np.median(dd_grid)),
                     "grid_p90": float(np.percentile(dd_grid, 90))},
        "gradient_vs_grid": {"within_1e-9s": float(np.mean(gg_p <= 1e-9)),
                             "within_0.01dm": float(np.mean(gg_d <= 0.01)),
                             "period_median_s": float(np.median(gg_p)),
                             "dm_median": float(np.median(gg_d)),
                             "grid_period_step_median_s": float(p_quant),
                             "grid_dm_half_step": float(step / 2)},
        "fine_grid": {"s_per_candidate": round(t_fine / ncand, 6),
                      "period_error_median_s": float(np.median(dp_fine)),
                      "dm_error_median": float(np.median(dd_fine)),
                      "gradient_within_1e-9s": float(np.mean(gf_p <= 1e-9)),
                      "gradient_within_0.01dm": float(np.mean(gf_d <= 0.01)),
                      "gradient_vs_fine_period_median_s": float(np.median(gf_p)),
                      "gradient_vs_fine_dm_median": float(np.median(gf_d))},
    }
    print(json.dumps(line))


# ------------------------------------------------------------ survey scale
SURVEY_RFI = dict(nb_channels=41, nb_amplitude=48.0, nb_hz=50.0, nbursts=10,
                  burst_samples=781, burst_amplitude=32.0)


def survey_observation(ns=1 << 23, seed=5):
    """The survey-scale observation, generated on the device: 4096 ch x 8-bit
    at 64 us, 1200-1600 MHz, noise N(128, 16) with +-10% channel gains, 20
    seeded pulsars (P 1 ms - 4 s log-uniform, DM 5-2500, duty 2-6%), then
    narrowband RFI (41 channels, a 50 Hz modulation of 3 sigma) and 10
    broadband bursts (0.05 s, 2 sigma)."""
    from pulsarsr_gb300 import synth
    rng = np.random.default_rng(seed)
    nch, tsamp, fch1, foff = 4096, 64e-6, 1600.0, -400.0 / 4096
    pulsars = [synth.Pulsar(float(np.exp(rng.uniform(np.log(0.001), np.log(4.0)))),
                            float(rng.uniform(5, 2500)), float(rng.uniform(0.02, 0.06)),
                            float(rng.uniform(0.01, 0.04)), phase=float(rng.uniform(0, 1)))
               for _ in range(20)]
    fb = synth.device(nch, 8, ns, tsamp, fch1, foff, seed=seed, noise_mean=128.0,
                      noise_sigma=16.0, gain_spread=0.1, pulsars=pulsars)
    synth.inject_rfi(fb, seed, **SURVEY_RFI)
    return fb, pulsars, tsamp


def survey_cpu_subset(trials, cfg_kw, ntrials=16):
    """The oracle on the host cores at the survey's channel count: a
    4096-channel 2^19-sample observation from the same generator (8.6 GB as
    f32 on the host), RFI mask, then `ntrials` trial DMs spread over the
    plan; the rate is per DM-trial*sample (a subset, stated as such)."""
    from oracle import oracle as O
    O.build()
    from pulsarsr_gb300 import dedisperse
    fb, _, tsamp = survey_observation(ns=1 << 19)
    freqs = fb.header.frequencies()
    d = fb.data
    fb.close()
    md = int(dedisperse.delays(freqs, tsamp, float(trials[-1])).max())
    disc = ((1 << 19) - 2 * md) // 2
    pick = trials[np.linspace(0, len(trials) - 1, ntrials).round().astype(int)]
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    m, _ = O.rfi_mask(d, max(int(0.1 / tsamp), 32), 8.0)
    t_rfi = time.perf_counter() - t0
    del d
    t0 = time.perf_counter()
    O.search_trials(m, freqs, tsamp, pick, disc, threads=threads, **cfg_kw)
    t_tr = time.perf_counter() - t0
    return {"value": round(ntrials * disc / t_tr, 1), "unit": UNIT, "cores": threads,
            "kind": "port",
            "sample": f"4096 ch x 8-bit x 2^19 samples (same generator), RFI mask "
                      f"({t_rfi:.1f}s), then {ntrials} of the plan's {len(trials)} trials "
                      f"(discovery {disc}) in {t_tr:.1f}s on {threads} threads; rate per "
                      "DM-trial*sample, extrapolated to the full observation"}


def run_survey(args):
    """The survey-scale search (survey_observation): RFI masking, 8000 trials
    over DM 0-3000 (step 0.37504) in 256-trial HBM blocks, rFFT 2^23,
    harmonic sums to 32 (one level beyond the reference's 16), then gradient
    refinement of the 512 highest-scoring sifted candidates."""
    from pulsarsr_gb300 import dedisperse, fold, rfi, search
    rt = cudart()
    nch, ns = 4096, 1 << 23
    t0 = time.perf_counter()
    fb, pulsars, tsamp = survey_observation(ns)
    rt.cudaDeviceSynchronize()
    t_synth = time.perf_counter() - t0
    freqs = fb.header.frequencies()
    trials = dedisperse.plan(0.0, 3000.0, 0.37504)
    md = int(dedisperse.delays(freqs, tsamp, 3000.0).max())
    discovery = (ns - 2 * md) // 2
    cfg = search.Config(min_hz=15.0, max_hz=2000.0, threshold=8.0, max_candidates=32,
                        max_harmonics=32)
    block = max(int(0.1 / tsamp), 32)
    rt.cudaDeviceSynchronize()
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    mask = rfi.mask(fb, block, 8.0)
    counts, cands = search.search_trials(fb, trials, discovery, cfg)
    rt.cudaDeviceSynchronize()
    t_search = time.perf_counter() - t0
    clk = clocks.stop()
    # search::sift (search/src/lib.rs:147-176): harmonic and duplicate
    # families collapsed, zero-DM candidates rejected, best 512 kept.
    top = search.sift(cands, 1.0 / (discovery * tsamp), 512, True)
    starts = [(float(c["period_s"]), 0.0, float(c["dm"])) for c in top]
    n = ns - md - 4
    t0 = time.perf_counter()
    fold.refine_gradient(fb, n, starts, dm_window=10 * 0.37505 / 2)
    rt.cudaDeviceSynchronize()
    t_refine = time.perf_counter() - t0
    units = len(trials) * discovery
    # An injected pulsar is recovered when a sifted candidate lies within two
    # bins of one of its harmonics m f0 or sub-harmonics f0 / m (m <= 32) and
    # within 20 of its DM; pulsars slower than min_hz appear only through
    # their harmonics.
    res = 1.0 / (discovery * tsamp)
    found, recovered = 0, []
    for p in pulsars:
        f = 1.0 / p.period_s
        hit = any(abs(c["dm"] - p.dm) < 20 and
                  any(abs(c["frequency_hz"] - f * m) < 2 * res * m or
                      abs(c["frequency_hz"] * m - f) < 2 * res * m for m in range(1, 33))
                  for c in top)
        found += int(hit)
        recovered.append({"period_s": round(p.period_s, 6), "dm": round(p.dm, 2),
                          "amplitude": round(p.amplitude, 4), "found": bool(hit)})
    cpu = None if args.no_cpu else survey_cpu_subset(
        trials, dict(min_hz=15.0, max_hz=2000.0, threshold=8.0, max_candidates=32,
                     max_harmonics=32))
    line = {
        "metric": "survey search DM-trial*samples/s (4096 ch, 8000 trials)",
        "value": round(units / t_search, 1), "unit": "DM-trial*samples/s", "n_gpus": 1,
        "higher_is_better": True, "dtype": "u8/f32", "data": "synthetic, generated on the device",
        "config": {"workload": "4096 ch x 8-bit x 2^23 samples, 64 us, 1200-1600 MHz, 20 pulsars, "
                               "narrowband + burst RFI; DM 0-3000 step 0.37504 (8000 trials), "
                               "discovery "
                               f"{discovery}, rFFT {2 * (1 << (discovery - 1).bit_length())}, "
                               "harmonic sums to 32, RFI on",
                   "trials": len(trials), "discovery_samples": int(discovery)},
        "search_seconds": round(t_search, 3), "synth_seconds": round(t_synth, 3),
        "refine_seconds": round(t_refine, 3),
        "masked_fraction": mask.masked_fraction, "candidates": int(len(cands)),
        "sifted": int(len(top)), "injected_pulsars_in_sifted": found,
        "injected": recovered,
        "rfi": {"injected": SURVEY_RFI, "channels_masked": len(mask.channels),
                "blocks_masked": len(mask.blocks)},
        "h32_candidates": int((cands["harmonics"] == 32).sum()),
        "clocks": clk,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line))


# ------------------------------------------------------------ cube fold
def run_fold(args):
    """The cube fold of gradient refinement by regime: 256 ch x 8-bit x 2^23
    samples (2.1 GB, larger than L2) at 64 us with three pulsars, each refined
    alone with one evaluation (fold, row DFTs, one objective + adjoint) at 128
    bins x 64 subints.  P 0.794 s: 0.010 bins per sample (8-bit run sums);
    P 24.04 ms: 0.34 (bin-owner gather); P 2.04 ms: 4.0 (per-sample scatter)."""
    from pulsarsr_gb300 import dedisperse, fold, synth
    rt = cudart()
    nch, ns, tsamp, fch1, foff = 256, 1 << 23, 64e-6, 1600.0, -400.0 / 256
    regimes = [("slow", 0.79372, 2020.8), ("walk", 0.02404, 1024.1), ("fast", 0.00204, 2113.1)]
    pulsars = [synth.Pulsar(P, dm, 0.04, 0.03, phase=0.3) for _, P, dm in regimes]
    fb = synth.device(nch, 8, ns, tsamp, fch1, foff, seed=5, noise_mean=128.0,
                      noise_sigma=16.0, gain_spread=0.1, pulsars=pulsars)
    md = int(dedisperse.delays(fb.header.frequencies(), tsamp, 3000.0).max())
    n = ns - md - 4
    out = {}
    for name, P, dm in regimes:
        start = [(P * (1 + 1e-7), 0.0, dm + 0.3)]
        for _ in range(max(args.warmup, 1)):
            fold.refine_gradient(fb, n, start, max_evals=1)
        rt.cudaDeviceSynchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            fold.refine_gradient(fb, n, start, max_evals=1)
        rt.cudaDeviceSynchronize()
        ms = (time.perf_counter() - t0) / args.steps * 1e3
        out[name] = {"period_s": P, "bins_per_sample": round(128 * tsamp / P, 4),
                     "ms_per_refine": round(ms, 4),
                     "effective_GBps": round(nch * n / (ms * 1e-3) / 1e9, 1)}
    line = {"metric": "cube fold + one evaluation, ms per call", "unit": "ms",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": False, "dtype": "u8 data, f32 bins, fixed-point phases",
            "data": "synthetic, generated on the device",
            "config": {"workload": "256 ch x 8-bit x 2^23 samples (2.1 GB), 64 us, 128 bins x "
                                   "64 subints, one start per regime", "n": int(n)},
            "regimes": out}
    print(json.dumps(line))


# ------------------------------------------------------------ batch
def run_batch(args):
    """64 seeded observations of uneven shape searched by one CUDA graph:
    channels from {64, 128, 256, 512, 1024}, 8-bit, 2^18-2^22 samples
    (log-uniform), tsamp 64-256 us, 1200-1600 MHz, 200-4000 trials at the
    default DM step, 0-2 pulsars (P 1.5 ms-2 s, DM 10-800 within the plan,
    folded SNR 8-40), generated on the device; RFI masking on."""
    from pulsarsr_gb300 import batch, dedisperse, fbank, search, synth
    rt = cudart()
    rng = np.random.default_rng(3)
    cfg = search.Config(min_hz=1.0, max_hz=2000.0, threshold=8.0, max_candidates=32)
    specs, obs = [], []
    for i in range(64):
        nch = int(rng.choice([64, 128, 256, 512, 1024]))
        ns = int(np.exp(rng.uniform(np.log(1 << 18), np.log(1 << 22))))
        tsamp = float(rng.uniform(64e-6, 256e-6))
        fch1, foff = 1600.0, -400.0 / nch
        freqs = fch1 + np.arange(nch) * foff
        step = dedisperse.dm_step(freqs, tsamp)
        nt = int(rng.integers(200, 4001))
        dm_max = step * (nt - 1)
        trials = dedisperse.plan(0.0, dm_max, step)
        md = int(dedisperse.delays(freqs, tsamp, float(trials[-1])).max())
        disc = (ns - 2 * md) // 2
        ps = []
        for _ in range(int(rng.integers(0, 3))):
            P = float(np.exp(rng.uniform(np.log(0.0015), np.log(2.0))))
            duty = float(rng.uniform(0.02, 0.06))
            snr = float(rng.uniform(8, 40))
            amp = snr / np.sqrt(nch * ns * duty)
            ps.append(synth.Pulsar(P, float(rng.uniform(10, min(800.0, float(trials[-1])))),
                                   duty, float(amp), phase=float(rng.uniform(0, 1))))
        specs.append((nch, ns, tsamp, fch1, foff, ps))
        h = fbank.HeaderInfo(nch, 8, tsamp, fch1, foff, 0)
        obs.append(dict(header=h, nsamples=ns, trials=trials, discovery=disc, config=cfg,
                        rfi_block=max(int(0.1 / tsamp), 32), rfi_threshold=8.0))
    b = batch.Batch(obs, hbm_budget_bytes=64 << 30)
    for i, (nch, ns, tsamp, fch1, foff, ps) in enumerate(specs):
        fb = synth.device(nch, 8, ns, tsamp, fch1, foff, seed=300 + i, noise_mean=128.0,
                          noise_sigma=16.0, pulsars=ps)
        b.load_fb(i, fb)
        del fb
    units = sum(len(o["trials"]) * o["discovery"] for o in obs)
    ev = Events(rt)

    def timed(k):
        out = []
        for _ in range(k):
            rt.cudaDeviceSynchronize()
            a, e = ev.new(), ev.new()
            ev.record(a, b.stream)
            b.run()
            ev.record(e, b.stream)
            out.append(ev.ms(a, e))
            b.sync()
        return statistics.mean(out)

    b.run()  # warm-up + graph capture
    b.sync()
    ms_default = timed(max(args.steps // 3, 2))
    t0 = time.perf_counter()
    chunk, inner, subbands = b.tune()
    t_tune = time.perf_counter() - t0
    b.run()
    b.sync()
    clocks = ClockSampler(0)
    clocks.start()
    ms_tuned = timed(max(args.steps // 3, 2))
    clk = clocks.stop()
    adds = sum(len(o["trials"]) * o["discovery"] * o["header"].nchans for o in obs)
    line = {
        "metric": "batched search DM-trial*samples/s (64 uneven observations, one graph)",
        "value": round(units / (ms_tuned / 1e3), 1), "unit": "DM-trial*samples/s", "n_gpus": 1,
        "higher_is_better": True, "dtype": "u8/f32", "data": "synthetic, generated on the device",
        "config": {"workload": "64 observations: 64-1024 ch, 8-bit, 2^18-2^22 samples, "
                               "64-256 us, 200-4000 trials each, 0-2 pulsars, RFI on",
                   "dm_trial_samples": int(units), "channel_adds": int(adds),
                   "timing": "CUDA events around one graph launch on the batch stream"},
        "ms_per_batch_untuned": round(ms_default, 3), "ms_per_batch_tuned": round(ms_tuned, 3),
        "tune_seconds": round(t_tune, 2),
        "tuned_dm_block": {str(int(k)): int(v) for k, v in
                           zip(*np.unique(chunk, return_counts=True))},
        "tuned_fft_chunk": {str(int(k)): int(v) for k, v in
                            zip(*np.unique(inner, return_counts=True))},
        "tuned_subbands": {str(int(k)): int(v) for k, v in
                           zip(*np.unique(subbands, return_counts=True))},
        "clocks": clk,
    }
    if not args.no_cpu:
        line["cpu_baseline"] = batch_cpu_sample(specs, obs)
    print(json.dumps(line))


def batch_cpu_sample(specs, obs, every=16, ntrials=32):
    """The oracle on the host cores for the batch: every `every`-th
    observation regenerated with the same generator, RFI-masked, and
    `ntrials` of its trial DMs spread over its plan searched on all threads;
    the rate is the sampled DM-trial*samples over the summed time (a subset,
    stated as such)."""
    from oracle import oracle as O
    O.build()
    from pulsarsr_gb300 import synth
    threads = os.cpu_count() or 1
    units, secs, picked = 0, 0.0, []
    for i in range(0, len(specs), every):
        nch, ns, tsamp, fch1, foff, ps = specs[i]
        o = obs[i]
        fb = synth.device(nch, 8, ns, tsamp, fch1, foff, seed=300 + i, noise_mean=128.0,
                          noise_sigma=16.0, pulsars=ps)
        d = fb.data
        fb.close()
        freqs = fch1 + np.arange(nch) * foff
        t0 = time.perf_counter()
        m, _ = O.rfi_mask(d, o["rfi_block"], 8.0)
        t_rfi = time.perf_counter() - t0
        del d
        tr = o["trials"]
        pick = tr[np.linspace(0, len(tr) - 1, min(ntrials, len(tr))).round().astype(int)]
        t0 = time.perf_counter()
        O.search_trials(m, freqs, tsamp, pick, o["discovery"], threads=threads, min_hz=1.0,
                        max_hz=2000.0, threshold=8.0, max_candidates=32)
        t_tr = time.perf_counter() - t0
        # the whole observation: RFI once plus every trial at the sampled rate
        secs += t_rfi + t_tr * len(tr) / len(pick)
        units += len(tr) * o["discovery"]
        picked.append(f"{nch}ch x {ns} ({len(pick)} of {len(tr)} trials)")
    return {"value": round(units / secs, 1), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{len(picked)} of the {len(specs)} observations: "
                      f"{'; '.join(picked)}; each RFI-masked once, the trial time extrapolated "
                      f"from the sampled trials to its plan; {threads} threads"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c4", "c5", "fold"],
                    help="c1/c2: searches; c3: batch of 64 observations; c4: gradient vs "
                         "grid refinement; c5: survey scale; fold: the refinement cube "
                         "fold by regime")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--trials", type=int, default=0,
                    help="search only the first N trial DMs (small profiling case)")
    args = ap.parse_args()
    if args.config == "c3" and args.impl == "ours":
        # 64 concurrent graph branches: 32 hardware work queues instead of the
        # default 8 (read when the CUDA context is created, so set before any
        # CUDA call) measured 5.64 against 5.72 s per batch.
        os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    if args.impl == "reference":
        run_reference(args)
    else:
        from pulsarsr_gb300 import build
        build.build()
        if args.config == "c4":
            run_refine(args)
        elif args.config == "c5":
            run_survey(args)
        elif args.config == "c3":
            run_batch(args)
        elif args.config == "fold":
            run_fold(args)
        else:
            run_ours(args)


if __name__ == "__main__":
    main()
