// The trial loop of `psr search` (cli/src/main.rs:462-473) on the device:
// for a chunk of trial DMs, dedisperse -> FFT power -> normalise -> harmonic
// sums -> per-trial candidate lists, with every buffer allocated once.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "search.h"

namespace psr {

int SearchEngine::prepare(const DeviceObs &o, const double *trials, uint64_t ntrials_,
                          uint64_t n_, const SpecConfig &cfg, cudaStream_t st) {
  if (ntrials_ == 0) {
    set_error("search: empty DM plan");
    return PSR_EINVAL;
  }
  ntrials = ntrials_;
  n = n_;
  spec = cfg;
  nch = o.nch;
  std::vector<uint32_t> tab;
  uint64_t maxd = 0;
  PSR_TRY(make_delay_table(o, trials, ntrials, tab, max_spread, maxd));
  if (n < 2 || n > o.ns - maxd) {
    set_error("invalid dedispersion input: invalid output length");
    return PSR_EDEDISPERSE;
  }
  PSR_TRY(delays.ensure(tab.size() * 4));
  PSR_CUDA(cudaMemcpyAsync(delays.p, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice, st));
  PSR_TRY(trial_dm.ensure(ntrials * 8));
  PSR_CUDA(cudaMemcpyAsync(trial_dm.p, trials, ntrials * 8, cudaMemcpyHostToDevice, st));
  PSR_TRY(fft.init(n, st));
  ldo = series_ld(n);
  ldp = ((fft.M + 1 + 63) / 64) * 64;
  if (chunk == 0) chunk = 256;
  chunk = std::min(chunk, ntrials);
  if (inner == 0) {
    const uint64_t per = fft.m > 12 ? fft.M * 8 : 1;  // FFT work buffer per trial
    inner = std::max<uint64_t>(1, (4ull << 30) / per);
  }
  inner = std::min(inner, chunk);
  nparts = dedisperse_part_count(o, n);
  npsum = (uint32_t)fft.pass2_ctas();
  PSR_TRY(series.ensure(chunk * ldo * 4 + 256));
  PSR_TRY(parts.ensure(chunk * nparts * 8));
  PSR_TRY(sums.ensure(chunk * 8));
  PSR_TRY(means.ensure(chunk * 4));
  PSR_TRY(work.ensure(fft.m > 12 ? inner * fft.M * 8 : 16));
  PSR_TRY(power.ensure(2 * chunk * ldp * 4));
  PSR_TRY(psum.ensure(2 * chunk * npsum * 8));
  PSR_TRY(spectrum_prepare(fft, spec, chunk, inner, sw, st));
  const uint64_t maxc = std::max<uint64_t>(cfg.max_candidates, 1);
  PSR_TRY(kept.ensure(ntrials * maxc * sizeof(psr_candidate)));
  PSR_TRY(kept_count.ensure(ntrials * 4));
  PSR_TRY(err.ensure(16));
  PSR_CUDA(cudaMemsetAsync(err.p, 0, 16, st));
  const uint64_t tail = chunk >= 16 && ntrials > chunk ? chunk / 8 : 0;
  cstart.clear();
  for (uint64_t t = 0; t < ntrials - tail; t += chunk) cstart.push_back(t);
  if (tail) cstart.push_back(ntrials - tail);
  cstart.push_back(ntrials);
  nchunks = cstart.size() - 1;
  const int G = subbands >= 0 ? subbands : dedisp_subbands_default(o);
  PSR_TRY(build_subband_plan(tab, o.nch, cstart, o.kind == SAMPLE_U8 ? G : 0, sbplan, st));
  PSR_TRY(chunk_overflow.ensure(nchunks * 4 + 16));
  if (!aux) PSR_CUDA(cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking));
  for (cudaEvent_t *e : {&ev_fft[0], &ev_fft[1], &ev_sel[0], &ev_sel[1]})
    if (!*e) PSR_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  sel_pending[0] = sel_pending[1] = false;
  return PSR_OK;
}

int SearchEngine::enqueue_chunk(const DeviceObs &o, uint64_t ci, cudaStream_t st) {
  const uint64_t t0 = cstart[ci];
  const uint64_t nt = cstart[ci + 1] - t0;
  PSR_TRY(record(ST_DEDISP, true, st));
  PSR_TRY(launch_dedisperse_ex(o, delays.as<uint32_t>() + t0 * o.nch, nt, n, series.as<float>(),
                               ldo, parts.as<double>(), sums.as<double>(), means.as<float>(),
                               max_spread, err.as<unsigned>(), st, 0, 0, true, &sbplan, ci));
  PSR_TRY(record(ST_DEDISP, false, st));
  // aux runs after everything st has queued so far (the previous chunk's
  // work is ordered on aux already), then resets the candidate queues.
  PSR_CUDA(cudaEventRecord(ev_fft[1], st));
  PSR_CUDA(cudaStreamWaitEvent(aux, ev_fft[1], 0));
  PSR_TRY(spectrum_reset(sw, nt, aux));
  // This chunk's half of the power and psum buffers is rewritten below: the
  // selection of the chunk that used it last must be done with it.
  const int b = (int)(ci & 1);
  float *pw = power.as<float>() + (uint64_t)b * chunk * ldp;
  double *ps = psum.as<double>() + (uint64_t)b * chunk * npsum;
  if (sel_pending[b]) PSR_CUDA(cudaStreamWaitEvent(st, ev_sel[b], 0));
  uint64_t k = 0;
  for (uint64_t i0 = 0; i0 < nt; i0 += inner, ++k) {
    const uint64_t ni = std::min(inner, nt - i0);
    PSR_TRY(record(ST_FFT, true, st));
    PSR_TRY(launch_raw_power_ex(fft, series.as<float>() + i0 * ldo, ldo, means.as<float>() + i0,
                                ni, work.as<float2>(), pw + i0 * ldp, ldp, ps + i0 * npsum, st));
    PSR_TRY(record(ST_FFT, false, st));
    cudaEvent_t e = ev_fft[k & 1];
    PSR_CUDA(cudaEventRecord(e, st));
    PSR_CUDA(cudaStreamWaitEvent(aux, e, 0));
    PSR_TRY(record(ST_SPEC, true, aux));
    PSR_TRY(spectrum_gate(fft, spec, pw + i0 * ldp, ldp, ps + i0 * npsum, npsum, ni, i0, sw,
                          aux));
    PSR_TRY(record(ST_SPEC, false, aux));
  }
  const uint64_t maxc = std::max<uint64_t>(spec.max_candidates, 1);
  PSR_TRY(record(ST_SPEC, true, aux));
  PSR_TRY(spectrum_items(fft, spec, pw, ldp, nt, sw, aux));
  PSR_TRY(spectrum_select(fft, spec, trial_dm.as<double>() + t0, nt, sw,
                          kept.as<psr_candidate>() + t0 * maxc, kept_count.as<unsigned>() + t0,
                          aux));
  PSR_TRY(record(ST_SPEC, false, aux));
  PSR_CUDA(cudaMemcpyAsync(chunk_overflow.as<unsigned>() + ci, sw.overflow.p, 4,
                           cudaMemcpyDeviceToDevice, aux));
  PSR_CUDA(cudaEventRecord(ev_sel[b], aux));
  sel_pending[b] = true;
  if (profile == 2) PSR_CUDA(cudaStreamWaitEvent(st, ev_sel[b], 0));
  return PSR_OK;
}

int SearchEngine::join(cudaStream_t st) {
  for (int b = 0; b < 2; ++b) {
    if (sel_pending[b]) PSR_CUDA(cudaStreamWaitEvent(st, ev_sel[b], 0));
    sel_pending[b] = false;
  }
  return PSR_OK;
}

int SearchEngine::record(int stage, bool begin, cudaStream_t st) {
  if (!profile) return PSR_OK;
  cudaEvent_t e;
  PSR_CUDA(cudaEventCreate(&e));
  PSR_CUDA(cudaEventRecord(e, st));
  (begin ? ev_begin : ev_end)[stage].push_back(e);
  if (!begin) stage_launches[stage] += 1;
  return PSR_OK;
}

int SearchEngine::harvest() {
  for (int s = 0; s < ST_COUNT; ++s) {
    for (size_t i = 0; i < ev_begin[s].size() && i < ev_end[s].size(); ++i) {
      float ms = 0.0f;
      PSR_CUDA(cudaEventElapsedTime(&ms, ev_begin[s][i], ev_end[s][i]));
      stage_ms[s] += ms;
    }
    for (cudaEvent_t e : ev_begin[s]) cudaEventDestroy(e);
    for (cudaEvent_t e : ev_end[s]) cudaEventDestroy(e);
    ev_begin[s].clear();
    ev_end[s].clear();
  }
  return PSR_OK;
}

SearchEngine::~SearchEngine() {
  for (int s = 0; s < ST_COUNT; ++s) {
    for (cudaEvent_t e : ev_begin[s]) cudaEventDestroy(e);
    for (cudaEvent_t e : ev_end[s]) cudaEventDestroy(e);
  }
  for (cudaEvent_t e : {ev_fft[0], ev_fft[1], ev_sel[0], ev_sel[1]})
    if (e) cudaEventDestroy(e);
  if (aux) cudaStreamDestroy(aux);
}

int SearchEngine::enqueue(const DeviceObs &o, cudaStream_t st) {
  for (uint64_t ci = 0; ci < nchunks; ++ci) PSR_TRY(enqueue_chunk(o, ci, st));
  return join(st);
}

int SearchEngine::finish(const DeviceObs &o, cudaStream_t st) {
  // per-chunk overflow words, then the dedispersion error word
  PSR_TRY(h_status.ensure((nchunks + 1) * 4));
  unsigned *hs = h_status.as<unsigned>();
  PSR_CUDA(cudaMemcpyAsync(hs, chunk_overflow.p, nchunks * 4, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaMemcpyAsync(hs + nchunks, err.p, 4, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  std::vector<unsigned> ov(hs, hs + nchunks);
  const unsigned e = hs[nchunks];
  if (e) {
    set_error("dedispersion: a bounded wait for a staged tile gave up");
    return PSR_ETIMEOUT;
  }
  PSR_TRY(harvest());
  for (uint64_t ci = 0; ci < nchunks; ++ci) {
    int guard = 0;
    while (ov[ci]) {
      // Raw candidate storage overflowed for this chunk: grow it and redo.
      if (++guard > 8) {
        set_error("search: raw candidate storage overflow");
        return PSR_ECAPACITY;
      }
      sw.raw_cap *= 4;
      sw.queue_full = true;
      PSR_TRY(spectrum_prepare(fft, spec, chunk, inner, sw, st));
      PSR_TRY(enqueue_chunk(o, ci, st));
      PSR_TRY(join(st));
      unsigned v = 0;
      PSR_CUDA(cudaMemcpyAsync(&v, chunk_overflow.as<unsigned>() + ci, 4,
                               cudaMemcpyDeviceToHost, st));
      PSR_CUDA(cudaStreamSynchronize(st));
      ov[ci] = v;
    }
  }
  return PSR_OK;
}

int SearchEngine::collect(cudaStream_t st, uint64_t *counts, psr_candidate *out, uint64_t cap,
                          uint64_t *n_total) {
  const uint64_t maxc = std::max<uint64_t>(spec.max_candidates, 1);
  PSR_TRY(h_kept_count.ensure(ntrials * 4));
  PSR_TRY(h_kept.ensure(ntrials * maxc * sizeof(psr_candidate)));
  PSR_CUDA(cudaMemcpyAsync(h_kept_count.p, kept_count.p, ntrials * 4, cudaMemcpyDeviceToHost,
                           st));
  PSR_CUDA(cudaMemcpyAsync(h_kept.p, kept.p, ntrials * maxc * sizeof(psr_candidate),
                           cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  const unsigned *kc = h_kept_count.as<unsigned>();
  const psr_candidate *all = h_kept.as<psr_candidate>();
  uint64_t k = 0;
  for (uint64_t i = 0; i < ntrials; ++i) {
    if (counts) counts[i] = kc[i];
    // trial i's list, in order, as far as it fits
    if (out && k < cap) {
      const uint64_t m = std::min<uint64_t>(kc[i], cap - k);
      std::memcpy(out + k, all + i * maxc, m * sizeof(psr_candidate));
    }
    k += kc[i];
  }
  *n_total = k;
  if (out && k > cap) {
    set_error("search: candidate buffer too small (" + std::to_string(k) + " needed)");
    return PSR_ECAPACITY;
  }
  return PSR_OK;
}

}  // namespace psr

namespace psr {

// Delay tables in FP64 on the host (dedisperse/src/lib.rs:9-34).
int make_delay_table(const DeviceObs &o, const double *trials, uint64_t ntrials,
                     std::vector<uint32_t> &tab, uint64_t &max_spread, uint64_t &max_delay) {
  std::vector<double> freqs(o.nch);
  for (uint64_t c = 0; c < o.nch; ++c) freqs[c] = o.h.fch1 + (double)c * o.h.foff;
  tab.assign(ntrials * o.nch, 0);
  std::vector<uint64_t> d;
  max_delay = 0;
  for (uint64_t i = 0; i < ntrials; ++i) {
    if (!host_delays(freqs.data(), o.nch, o.h.tsamp, trials[i], d)) return PSR_EDEDISPERSE;
    for (uint64_t c = 0; c < o.nch; ++c) {
      max_delay = std::max(max_delay, d[c]);
      tab[i * o.nch + c] = (uint32_t)std::min<uint64_t>(d[c], 0xffffffffull);
    }
  }
  if (max_delay > o.ns) {
    set_error("invalid dedispersion input: delay exceeds observation");
    return PSR_EDEDISPERSE;
  }
  // Widest delay spread of any channel over any 8 consecutive trials (an
  // upper bound for every trial block of at most 8, whatever its alignment).
  max_spread = 0;
  for (uint64_t b = 0; b < ntrials; ++b)
    for (uint64_t c = 0; c < o.nch; ++c) {
      uint32_t lo = 0xffffffffu, hi = 0;
      for (uint64_t i = b; i < std::min<uint64_t>(b + 8, ntrials); ++i) {
        lo = std::min(lo, tab[i * o.nch + c]);
        hi = std::max(hi, tab[i * o.nch + c]);
      }
      max_spread = std::max<uint64_t>(max_spread, hi - lo);
    }
  return PSR_OK;
}

}  // namespace psr
