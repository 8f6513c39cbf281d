// confirmation::analyze (search/src/confirmation.rs:203-496) on the device.
//
// Host code drives device kernels only: every dedispersed series (the
// candidate-DM series, the 21-point half-step DM grid, the zero-DM control,
// the four subbands) is made by the dedispersion kernels into HBM and folded
// or measured there; the per-channel discovery profiles and the DM response
// are device kernels too.  What stays on the host is what the reference does
// on a few hundred numbers: grouping, window selection (64 x 5 candidate
// windows), the acceptance rules, and the JSON.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "analyze.h"
#include "search.h"

namespace psr {
namespace {

inline int64_t key64(double x) {
  int64_t i;
  std::memcpy(&i, &x, 8);
  return i ^ (int64_t)((uint64_t)(i >> 63) >> 1);
}

int dd_error(const std::string &what) {
  set_error("invalid dedispersion input: " + what);
  return PSR_EDEDISPERSE;
}

// A non-owning view of channels [c0, c1) of a device observation.
struct ChannelView {
  DeviceObs o;
  ChannelView(const DeviceObs &src, uint64_t c0, uint64_t c1) {
    o.h = src.h;
    o.h.nchans = (int64_t)(c1 - c0);
    o.h.fch1 = src.h.fch1 + (double)c0 * src.h.foff;
    o.ns = src.ns;
    o.nch = c1 - c0;
    o.kind = src.kind;
    o.ld = src.ld;
    o.samples.p = static_cast<unsigned char *>(src.samples.p) +
                  c0 * src.ld * (uint64_t)sample_bytes(src.kind);
    o.samples.bytes = 0;
  }
  ~ChannelView() { o.samples.p = nullptr; }
  ChannelView(const ChannelView &) = delete;
  ChannelView &operator=(const ChannelView &) = delete;
};

// Device dedispersion (dedisperse::apply, dedisperse/src/lib.rs:61-90) of
// ntr trials, tab[trial][channel] delays, n output samples each, into rows of
// stride ldo of `out`.
struct Dedisperser {
  DevBuf dd, out, parts, sums, means, err;
  uint64_t ldo = 0;
  int run(const DeviceObs &o, const std::vector<uint64_t> &tab, uint64_t ntr, uint64_t n,
          cudaStream_t st) {
    uint64_t maxd = 0;
    for (uint64_t d : tab) maxd = std::max(maxd, d);
    if (maxd > o.ns) return dd_error("delay exceeds observation");
    if (n < 2 || n > o.ns - maxd) return dd_error("invalid output length");
    std::vector<uint32_t> t32(tab.size());
    for (size_t i = 0; i < tab.size(); ++i) t32[i] = (uint32_t)tab[i];
    // Widest per-channel delay spread over any 8 consecutive trials.
    uint64_t spread = 0;
    for (uint64_t b = 0; b < ntr; ++b)
      for (uint64_t c = 0; c < o.nch; ++c) {
        uint32_t lo = 0xffffffffu, hi = 0;
        for (uint64_t i = b; i < std::min<uint64_t>(b + 8, ntr); ++i) {
          lo = std::min(lo, t32[i * o.nch + c]);
          hi = std::max(hi, t32[i * o.nch + c]);
        }
        spread = std::max<uint64_t>(spread, hi - lo);
      }
    ldo = series_ld(n);
    PSR_TRY(dd.ensure(t32.size() * 4));
    PSR_TRY(out.ensure(ntr * ldo * 4 + 256));
    PSR_TRY(parts.ensure(ntr * dedisperse_part_count(o, n) * 8 + 8));
    PSR_TRY(sums.ensure(ntr * 8));
    PSR_TRY(means.ensure(ntr * 4 + 4));
    PSR_TRY(err.ensure(8));
    PSR_CUDA(cudaMemsetAsync(err.p, 0, 8, st));
    PSR_CUDA(cudaMemcpyAsync(dd.p, t32.data(), t32.size() * 4, cudaMemcpyHostToDevice, st));
    PSR_TRY(launch_dedisperse_ex(o, dd.as<uint32_t>(), ntr, n, out.as<float>(), ldo,
                                 parts.as<double>(), sums.as<double>(), means.as<float>(),
                                 spread, err.as<unsigned>(), st, 0, 0, false));
    unsigned e = 0;
    PSR_CUDA(cudaMemcpyAsync(&e, err.p, 4, cudaMemcpyDeviceToHost, st));
    PSR_CUDA(cudaStreamSynchronize(st));
    if (e) {
      set_error("dedispersion: a bounded wait for a staged tile gave up");
      return PSR_ETIMEOUT;
    }
    return PSR_OK;
  }
  float *row(uint64_t i) const { return out.as<float>() + i * ldo; }
};

int delays_for(const std::vector<double> &freqs, double tsamp, double dm,
               std::vector<uint64_t> &d) {
  if (!host_delays(freqs.data(), freqs.size(), tsamp, dm, d)) return PSR_EDEDISPERSE;
  return PSR_OK;
}

// fold::profile_at of one device series.
int profile_dev(const float *d_x, uint64_t n, double tsamp, double period, uint64_t bins,
                uint64_t offset, FoldedProfile &p, cudaStream_t st) {
  p.values.resize(bins);
  p.counts.resize(bins);
  return fold_profiles(d_x, n, tsamp, &period, 1, bins, offset, &p.st, p.values.data(),
                       p.counts.data(), st);
}

// fold::refine (fold/src/lib.rs:81-97): max_by keeps the last maximum.
int refine_dev(const float *d_x, uint64_t n, double tsamp, double frequency, double span,
               uint64_t steps, uint64_t bins, FoldedProfile &best, cudaStream_t st) {
  if (!(steps > 0 && frequency > span && span >= 0.0)) {
    set_error("refine: steps > 0 and frequency > span_hz >= 0 required");
    return PSR_EINVAL;
  }
  std::vector<double> periods(steps + 1);
  for (uint64_t i = 0; i <= steps; ++i)
    periods[i] = 1.0 / (frequency - span + 2.0 * span * (double)i / (double)steps);
  std::vector<psr_profile_stats> sts(steps + 1);
  std::vector<float> vals((steps + 1) * bins);
  std::vector<uint64_t> cnts((steps + 1) * bins);
  PSR_TRY(fold_profiles(d_x, n, tsamp, periods.data(), steps + 1, bins, 0, sts.data(),
                        vals.data(), cnts.data(), st));
  uint64_t b = 0;
  for (uint64_t i = 1; i <= steps; ++i)
    if (key64(sts[i].reduced_chi_square) >= key64(sts[b].reduced_chi_square)) b = i;
  best.st = sts[b];
  best.values.assign(vals.begin() + b * bins, vals.begin() + (b + 1) * bins);
  best.counts.assign(cnts.begin() + b * bins, cnts.begin() + (b + 1) * bins);
  return PSR_OK;
}

// select_window (confirmation.rs:142-176): widths 1, 2, 4 .. bins/4, every
// start; the first strict maximum of the score wins.
psr_window select_window(const std::vector<float> &bins_v) {
  const uint64_t bins = bins_v.size();
  double best = -INFINITY;
  psr_window w{0, 1, bins};
  for (uint64_t width = 1; width <= bins / 4; width <<= 1) {
    for (uint64_t start = 0; start < bins; ++start) {
      double on = -0.0;
      for (uint64_t j = 0; j < width; ++j) on += (double)bins_v[(start + j) % bins];
      double total = -0.0;
      for (float v : bins_v) total += (double)v;
      const double contrast =
          on / (double)width - (total - on) / (double)(bins - width);
      const double score =
          contrast / std::sqrt(1.0 / (double)width + 1.0 / (double)(bins - width));
      if (score > best) {
        best = score;
        w = psr_window{start, width, bins};
      }
    }
  }
  return w;
}

int measure_dev(const float *d_x, uint64_t n, uint64_t offset, double tsamp, double period,
                const psr_window &w, psr_measurement &m, cudaStream_t st) {
  return measure_device(d_x, n, offset, tsamp, period, w.start_bin, w.width_bins, w.bins, &m,
                        st);
}

}  // namespace

int grid_refine_one(const DeviceObs &o, uint64_t n, const psr_timing &start,
                    double resolution, double dm_step, double dm_lo, double dm_hi,
                    uint64_t bins, psr_timing &out, double &rcs, cudaStream_t st) {
  std::vector<double> freqs(o.nch);
  for (uint64_t c = 0; c < o.nch; ++c) freqs[c] = o.h.fch1 + (double)c * o.h.foff;
  const double tsamp = o.h.tsamp;
  std::vector<uint64_t> d;
  PSR_TRY(delays_for(freqs, tsamp, start.dm, d));
  Dedisperser initial;
  PSR_TRY(initial.run(o, d, 1, n, st));
  FoldedProfile best;
  PSR_TRY(refine_dev(initial.row(0), n, tsamp, 1.0 / start.period_s, resolution, 40, bins,
                     best, st));
  double best_dm = start.dm;
  const double period = best.st.period_s;
  std::vector<double> dms(21);
  std::vector<uint64_t> grid;
  for (int i = -10; i <= 10; ++i) {
    const double dm = std::fmin(std::fmax(start.dm + (double)i * dm_step / 2.0, dm_lo), dm_hi);
    dms[(size_t)(i + 10)] = dm;
    PSR_TRY(delays_for(freqs, tsamp, dm, d));
    grid.insert(grid.end(), d.begin(), d.end());
  }
  Dedisperser g;
  PSR_TRY(g.run(o, grid, 21, n, st));
  std::vector<double> periods(21, period);
  std::vector<psr_profile_stats> sts(21);
  std::vector<float> vals(21 * bins);
  std::vector<uint64_t> cnts(21 * bins);
  PSR_TRY(fold_profiles_ex(g.row(0), g.ldo, n, tsamp, periods.data(), 21, bins, 0, sts.data(),
                           vals.data(), cnts.data(), st));
  for (size_t i = 0; i < 21; ++i)
    if (sts[i].reduced_chi_square > best.st.reduced_chi_square) {
      best.st = sts[i];
      best_dm = dms[i];
    }
  out.period_s = period;
  out.pdot = start.pdot;
  out.dm = best_dm;
  rcs = best.st.reduced_chi_square;
  return PSR_OK;
}

std::vector<Family> group_candidates(const psr_candidate *c, uint64_t n, double resolution,
                                     uint64_t limit, std::vector<uint64_t> *order,
                                     std::vector<int64_t> *family) {
  std::vector<uint64_t> idx(n);
  for (uint64_t i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) {
    return key64(c[a].score) > key64(c[b].score);
  });
  std::vector<Family> fams;
  if (order) order->assign(idx.begin(), idx.end());
  if (family) family->assign(n, -1);
  for (uint64_t k = 0; k < n; ++k) {
    const psr_candidate &x = c[idx[k]];
    int64_t found = -1;
    for (size_t f = 0; f < fams.size() && found < 0; ++f) {
      const psr_candidate &a = fams[f].leader;
      for (int h = 1; h <= 16; ++h)
        if (std::fabs(a.frequency_hz - x.frequency_hz * (double)h) <= resolution ||
            std::fabs(x.frequency_hz - a.frequency_hz * (double)h) <= resolution) {
          found = (int64_t)f;
          break;
        }
    }
    if (found >= 0) {
      fams[(size_t)found].members.push_back(x);
    } else if (fams.size() < limit) {
      found = (int64_t)fams.size();
      fams.push_back(Family{x, {x}});
    }
    if (family) (*family)[k] = found;
  }
  return fams;
}

int analyze_obs(const DeviceObs &o, const double *trials, uint64_t ntrials,
                const psr_candidate *generated, uint64_t ngenerated, uint64_t limit,
                uint64_t bins, const psr_rules &rules, Outcome &out, cudaStream_t st) {
  const uint64_t nch = o.nch, ns = o.ns;
  const double tsamp = o.h.tsamp;
  if (ntrials == 0 || !trials || limit == 0 || bins < 8 || nch < 4)
    return dd_error("confirmation requires >=4 channels, >=8 bins and valid array/trials");
  for (uint64_t i = 1; i < ntrials; ++i)
    if (!(trials[i] > trials[i - 1])) return dd_error("DM trials must increase");
  if (bins > 1024) {
    set_error("analyze: at most 1024 profile bins are supported");
    return PSR_EINVAL;
  }
  std::vector<double> freqs(nch);
  for (uint64_t c = 0; c < nch; ++c) freqs[c] = o.h.fch1 + (double)c * o.h.foff;
  const double max_dm = trials[ntrials - 1];
  std::vector<uint64_t> dmax;
  PSR_TRY(delays_for(freqs, tsamp, max_dm, dmax));
  const uint64_t guard = *std::max_element(dmax.begin(), dmax.end());
  if (guard > ns || ns - guard < 512) return dd_error("observation too short for confirmation");
  const uint64_t length = ns - guard;
  if (guard > length || length - guard < 256)
    return dd_error("DM delay leaves no independent split");
  const uint64_t discovery = (length - guard) / 2;
  const uint64_t vstart = discovery + guard;
  const uint64_t validation = length - vstart;
  const double resolution = 1.0 / ((double)discovery * tsamp);
  const double step = ntrials > 1 ? trials[1] - trials[0] : 1.0;

  out.rules = rules;
  out.info = psr_outcome_info{discovery, vstart, validation, length, ntrials, 0};
  out.candidates.clear();

  // Zero-DM discovery control (confirmation.rs:252-264).
  const std::vector<uint64_t> zeros(nch, 0);
  std::vector<psr_candidate> zero_c;
  {
    SpecConfig zc;
    zc.tsamp = tsamp;
    zc.min_hz = 1.0;
    zc.max_hz = 0.5 / tsamp;
    zc.threshold = 8.0;
    zc.max_candidates = 64;
    SearchEngine e;
    e.chunk = 1;
    const double zero_dm = 0.0;
    PSR_TRY(e.prepare(o, &zero_dm, 1, discovery, zc, st));
    PSR_TRY(e.enqueue(o, st));
    PSR_TRY(e.finish(o, st));
    uint64_t cnt = 0, total = 0;
    zero_c.resize(64);
    PSR_TRY(e.collect(st, &cnt, zero_c.data(), zero_c.size(), &total));
    zero_c.resize(total);
  }

  // Shared by every family: the full-length zero-DM series, the delay table of
  // every trial (DM response).
  Dedisperser zero;
  PSR_TRY(zero.run(o, zeros, 1, length, st));
  std::vector<uint32_t> tab;
  uint64_t tab_spread = 0, tab_max = 0;
  PSR_TRY(make_delay_table(o, trials, ntrials, tab, tab_spread, tab_max));
  DevBuf d_tab;
  PSR_TRY(d_tab.ensure(tab.size() * 4));
  PSR_CUDA(cudaMemcpyAsync(d_tab.p, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice, st));

  const std::vector<Family> fams = group_candidates(generated, ngenerated, resolution * 1.5,
                                                    limit);
  for (const Family &fam : fams) {
    const psr_candidate &cand = fam.leader;
    Confirmed r;
    r.members = fam.members;
    // Rational-frequency aliases of a zero-DM emitter (confirmation.rs:267-280).
    double zero_ratio = 0.0;
    for (const psr_candidate &z : zero_c) {
      bool rel = false;
      for (int m = 1; m <= 16 && !rel; ++m)
        for (int n = 1; n <= 16 && !rel; ++n)
          rel = std::fabs(cand.frequency_hz - z.frequency_hz * (double)m / (double)n) <=
                resolution * 1.5;
      if (rel) zero_ratio = std::fmax(zero_ratio, z.score / std::fmax(cand.score, 1.0));
    }
    std::vector<uint64_t> d;
    PSR_TRY(delays_for(freqs, tsamp, cand.dm, d));
    Dedisperser initial;
    PSR_TRY(initial.run(o, d, 1, length, st));
    FoldedProfile best;
    PSR_TRY(refine_dev(initial.row(0), discovery, tsamp, cand.frequency_hz, resolution, 40,
                       bins, best, st));
    double best_dm = cand.dm;
    const double period = best.st.period_s;
    // Half-step DM grid at the refined period (confirmation.rs:295-310).
    {
      std::vector<double> dms(21);
      std::vector<uint64_t> grid;
      for (int i = -10; i <= 10; ++i) {
        const double dm =
            std::fmin(std::fmax(cand.dm + (double)i * step / 2.0, trials[0]), max_dm);
        dms[(size_t)(i + 10)] = dm;
        PSR_TRY(delays_for(freqs, tsamp, dm, d));
        grid.insert(grid.end(), d.begin(), d.end());
      }
      Dedisperser g;
      PSR_TRY(g.run(o, grid, 21, discovery, st));
      std::vector<double> periods(21, period);
      std::vector<psr_profile_stats> sts(21);
      std::vector<float> vals(21 * bins);
      std::vector<uint64_t> cnts(21 * bins);
      PSR_TRY(fold_profiles_ex(g.row(0), g.ldo, discovery, tsamp, periods.data(), 21, bins, 0,
                               sts.data(), vals.data(), cnts.data(), st));
      for (size_t i = 0; i < 21; ++i)
        if (sts[i].reduced_chi_square > best.st.reduced_chi_square) {
          best.st = sts[i];
          best.values.assign(vals.begin() + i * bins, vals.begin() + (i + 1) * bins);
          best.counts.assign(cnts.begin() + i * bins, cnts.begin() + (i + 1) * bins);
          best_dm = dms[i];
        }
    }
    const psr_window window = select_window(best.values);
    PSR_TRY(delays_for(freqs, tsamp, best_dm, d));
    Dedisperser series;
    PSR_TRY(series.run(o, d, 1, length, st));
    psr_measurement vm{};
    PSR_TRY(measure_dev(series.row(0) + vstart, length - vstart, vstart, tsamp, period, window,
                        vm, st));
    // Zero-DM control refined in frequency and width (confirmation.rs:320-349).
    FoldedProfile zr;
    PSR_TRY(refine_dev(zero.row(0) + vstart, length - vstart, tsamp, 1.0 / period,
                       resolution * 2.0, 40, bins, zr, st));
    const double zero_period = zr.st.period_s;
    FoldedProfile zp;
    PSR_TRY(profile_dev(zero.row(0) + vstart, length - vstart, tsamp, zero_period, bins, vstart,
                        zp, st));
    const psr_window zw = select_window(zp.values);
    psr_measurement zm{};
    PSR_TRY(measure_dev(zero.row(0) + vstart, length - vstart, vstart, tsamp, zero_period, zw,
                        zm, st));
    const double contrast = std::fmax(vm.snr, 0.0) / std::fmax(zm.snr, 1.0);
    const double dispersion_widths =
        ((double)*std::max_element(d.begin(), d.end()) * tsamp) /
        (period * (double)window.width_bins / (double)bins);
    // Held-out time parts (confirmation.rs:354-361).
    for (uint64_t part = 0; part < 4; ++part) {
      const uint64_t lo = vstart + part * validation / 4;
      const uint64_t hi = vstart + (part + 1) * validation / 4;
      PSR_TRY(measure_dev(series.row(0) + lo, hi - lo, lo, tsamp, period, window,
                          r.s.time_parts[part], st));
      FoldedProfile tp;
      PSR_TRY(profile_dev(series.row(0) + lo, hi - lo, tsamp, period, bins, lo, tp, st));
      r.time_profiles[part] = tp.values;
    }
    // Subbands of nch/4 channels (confirmation.rs:362-390).
    for (uint64_t part = 0; part < 4; ++part) {
      const uint64_t lo = part * nch / 4, hi = (part + 1) * nch / 4;
      ChannelView view(o, lo, hi);
      std::vector<uint64_t> ds(d.begin() + lo, d.begin() + hi);
      Dedisperser sb;
      PSR_TRY(sb.run(view.o, ds, 1, length, st));
      PSR_TRY(measure_dev(sb.row(0) + vstart, length - vstart, vstart, tsamp, period, window,
                          r.s.subbands[part], st));
      FoldedProfile sp;
      PSR_TRY(profile_dev(sb.row(0) + vstart, length - vstart, tsamp, period, bins, vstart, sp,
                          st));
      r.subband_profiles[part] = sp.values;
    }
    // Per-channel first-half profiles and the DM response (confirmation.rs:391-433).
    std::vector<float> chp;
    PSR_TRY(fold_channels(o, discovery, tsamp, period, bins, chp, st));
    std::vector<double> chmean(nch);
    for (uint64_t c = 0; c < nch; ++c) {
      double m = -0.0;
      for (uint64_t b = 0; b < bins; ++b) m += (double)chp[c * bins + b];
      chmean[c] = m / (double)bins;
    }
    std::vector<double> comb;
    PSR_TRY(dm_response(chp, chmean, d_tab.as<uint32_t>(), ntrials, nch, bins, tsamp, period,
                        comb, st));
    r.dm_response.resize(ntrials);
    for (uint64_t ti = 0; ti < ntrials; ++ti) {
      const double *cb = comb.data() + ti * bins;
      double on = -0.0;
      for (uint64_t i = 0; i < window.width_bins; ++i) on += cb[(window.start_bin + i) % bins];
      on /= (double)window.width_bins;
      double tot = -0.0;
      for (uint64_t b = 0; b < bins; ++b) tot += cb[b];
      const double off =
          (tot - on * (double)window.width_bins) / (double)(bins - window.width_bins);
      DmPoint &p = r.dm_response[ti];
      p.dm = trials[ti];
      p.discovery_profile_response = on - off;
      // max_by over matching members keeps the last maximum.
      const psr_candidate *match = nullptr;
      for (const psr_candidate &c : r.members)
        if (std::fabs(c.dm - p.dm) < step * 0.01 &&
            std::fabs(c.frequency_hz - cand.frequency_hz) < resolution * 1.5)
          if (!match || key64(c.score) >= key64(match->score)) match = &c;
      if (match) {
        p.matched = true;
        p.spectral_score = match->score;
        p.spectral_frequency_hz = match->frequency_hz;
      }
    }
    // Acceptance rules (confirmation.rs:435-470).
    uint32_t mask = 0;
    if (vm.snr < rules.minimum_validation_snr) {
      mask |= 1u;
      r.reasons.push_back("held-out pulse SNR below threshold");
    }
    uint64_t np = 0, nsb = 0;
    for (const psr_measurement &m : r.s.time_parts) np += m.snr >= rules.minimum_part_snr;
    for (const psr_measurement &m : r.s.subbands) nsb += m.snr >= rules.minimum_part_snr;
    if (np < rules.minimum_time_parts) {
      mask |= 2u;
      r.reasons.push_back("pulse does not persist in enough held-out time segments");
    }
    if (nsb < rules.minimum_subbands) {
      mask |= 4u;
      r.reasons.push_back("pulse does not persist in enough held-out subbands");
    }
    if (best_dm <= 0.0 || contrast < rules.minimum_dm_contrast) {
      mask |= 8u;
      r.reasons.push_back("insufficient improvement over zero-DM interference control");
    }
    if (dispersion_widths < rules.minimum_dispersion_widths) {
      mask |= 16u;
      r.reasons.push_back(
          "dispersion sweep too small relative to selected pulse width to distinguish local "
          "interference");
    }
    if (zero_ratio > rules.maximum_zero_dm_spectral_ratio) {
      mask |= 32u;
      r.reasons.push_back(
          "stronger rationally related periodic signal in zero-DM discovery control");
    }
    r.s.candidate = cand;
    r.s.refined_dm = best_dm;
    r.s.profile = best.st;
    r.profile = best;
    r.s.window = window;
    r.s.validation = vm;
    r.s.zero_dm_validation = zm;
    r.s.zero_dm_period_s = zero_period;
    r.s.zero_dm_window = zw;
    r.s.dm_contrast = contrast;
    r.s.dispersion_widths = dispersion_widths;
    r.s.zero_dm_related_spectral_ratio = zero_ratio;
    r.s.harmonic_members = r.members.size();
    r.s.accepted = mask == 0;
    r.s.rejection_mask = mask;
    out.candidates.push_back(std::move(r));
  }
  out.info.candidates = out.candidates.size();
  return PSR_OK;
}

// ----------------------------------------------------------------- JSON
using psrjson::Value;

Value candidate_json(const psr_candidate &c) {
  Value v = Value::object();
  v.set("frequency_hz", Value::num(c.frequency_hz));
  v.set("period_s", Value::num(c.period_s));
  v.set("dm", Value::num(c.dm));
  v.set("harmonics", Value::u64(c.harmonics));
  v.set("score", Value::num(c.score));
  return v;
}

namespace {
Value measurement_json(const psr_measurement &m) {
  Value v = Value::object();
  v.set("snr", Value::num(m.snr));
  v.set("on_samples", Value::u64(m.on_samples));
  v.set("off_samples", Value::u64(m.off_samples));
  v.set("mean_difference", Value::num(m.mean_difference));
  v.set("standard_error", Value::num(m.standard_error));
  return v;
}
Value window_json(const psr_window &w) {
  Value v = Value::object();
  v.set("start_bin", Value::u64(w.start_bin));
  v.set("width_bins", Value::u64(w.width_bins));
  v.set("bins", Value::u64(w.bins));
  return v;
}
Value f32_array(const std::vector<float> &x) {
  Value a = Value::array();
  for (float f : x) a.push(Value::num32(f));
  return a;
}
}  // namespace

Value profile_json(const FoldedProfile &p) {
  Value v = Value::object();
  v.set("period_s", Value::num(p.st.period_s));
  v.set("snr", Value::num(p.st.snr));
  v.set("reduced_chi_square", Value::num(p.st.reduced_chi_square));
  v.set("bins", f32_array(p.values));
  Value c = Value::array();
  for (uint64_t x : p.counts) c.push(Value::u64(x));
  v.set("counts", std::move(c));
  return v;
}

Value confirmed_json(const Confirmed &r) {
  Value v = Value::object();
  v.set("candidate", candidate_json(r.s.candidate));
  v.set("refined_dm", Value::num(r.s.refined_dm));
  v.set("profile", profile_json(r.profile));
  v.set("window", window_json(r.s.window));
  v.set("validation", measurement_json(r.s.validation));
  v.set("zero_dm_validation", measurement_json(r.s.zero_dm_validation));
  v.set("zero_dm_period_s", Value::num(r.s.zero_dm_period_s));
  v.set("zero_dm_window", window_json(r.s.zero_dm_window));
  v.set("dm_contrast", Value::num(r.s.dm_contrast));
  v.set("dispersion_widths", Value::num(r.s.dispersion_widths));
  v.set("zero_dm_related_spectral_ratio", Value::num(r.s.zero_dm_related_spectral_ratio));
  Value tp = Value::array(), sb = Value::array(), tpr = Value::array(), sbr = Value::array();
  for (int i = 0; i < 4; ++i) {
    tp.push(measurement_json(r.s.time_parts[i]));
    sb.push(measurement_json(r.s.subbands[i]));
    tpr.push(f32_array(r.time_profiles[i]));
    sbr.push(f32_array(r.subband_profiles[i]));
  }
  v.set("time_parts", std::move(tp));
  v.set("subbands", std::move(sb));
  v.set("time_profiles", std::move(tpr));
  v.set("subband_profiles", std::move(sbr));
  Value resp = Value::array();
  for (const DmPoint &p : r.dm_response) {
    Value q = Value::object();
    q.set("dm", Value::num(p.dm));
    q.set("spectral_score", p.matched ? Value::num(p.spectral_score) : Value::null());
    q.set("spectral_frequency_hz",
          p.matched ? Value::num(p.spectral_frequency_hz) : Value::null());
    q.set("discovery_profile_response", Value::num(p.discovery_profile_response));
    resp.push(std::move(q));
  }
  v.set("dm_response", std::move(resp));
  Value mem = Value::array();
  for (const psr_candidate &c : r.members) mem.push(candidate_json(c));
  v.set("harmonic_members", std::move(mem));
  v.set("accepted", Value::boolean(r.s.accepted != 0));
  Value rs = Value::array();
  for (const std::string &s : r.reasons) rs.push(Value::str(s));
  v.set("rejection_reasons", std::move(rs));
  return v;
}

Value outcome_json(const Outcome &o) {
  Value rules = Value::object();
  rules.set("version", Value::str("split-confirm-v1"));
  rules.set("minimum_validation_snr", Value::num(o.rules.minimum_validation_snr));
  rules.set("minimum_part_snr", Value::num(o.rules.minimum_part_snr));
  rules.set("minimum_time_parts", Value::u64(o.rules.minimum_time_parts));
  rules.set("minimum_subbands", Value::u64(o.rules.minimum_subbands));
  rules.set("minimum_dm_contrast", Value::num(o.rules.minimum_dm_contrast));
  rules.set("minimum_dispersion_widths", Value::num(o.rules.minimum_dispersion_widths));
  rules.set("maximum_zero_dm_spectral_ratio", Value::num(o.rules.maximum_zero_dm_spectral_ratio));
  Value v = Value::object();
  v.set("rules", std::move(rules));
  v.set("discovery_samples", Value::u64(o.info.discovery_samples));
  v.set("validation_start_sample", Value::u64(o.info.validation_start_sample));
  v.set("validation_samples", Value::u64(o.info.validation_samples));
  v.set("common_samples", Value::u64(o.info.common_samples));
  v.set("trial_count", Value::u64(o.info.trial_count));
  Value c = Value::array();
  for (const Confirmed &r : o.candidates) c.push(confirmed_json(r));
  v.set("candidates", std::move(c));
  return v;
}

}  // namespace psr

// ------------------------------------------------------------------ C ABI
using namespace psr;

extern "C" {

void psr_rules_default(psr_rules *out) {
  if (!out) return;
  *out = psr_rules{6.0, 1.0, 3, 3, 1.25, 1.5, 1.0};
}

int psr_group(const psr_candidate *in, uint64_t n, double resolution_hz, uint64_t limit,
              uint64_t *order, int64_t *family, uint64_t *nfamilies) {
  if ((!in && n) || !nfamilies) {
    set_error("group: null argument");
    return PSR_EINVAL;
  }
  std::vector<uint64_t> ord;
  std::vector<int64_t> fam;
  const std::vector<Family> f = group_candidates(in, n, resolution_hz, limit, &ord, &fam);
  if (order) std::copy(ord.begin(), ord.end(), order);
  if (family) std::copy(fam.begin(), fam.end(), family);
  *nfamilies = f.size();
  return PSR_OK;
}

int psr_outcome_info_get(const psr_outcome *o, psr_outcome_info *out) {
  if (!o || !out) {
    set_error("outcome: null argument");
    return PSR_EINVAL;
  }
  *out = o->o.info;
  return PSR_OK;
}

int psr_outcome_candidate(const psr_outcome *o, uint64_t i, psr_confirmed *out,
                          float *profile_bins, uint64_t *profile_counts) {
  if (!o || !out || i >= o->o.candidates.size()) {
    set_error("outcome: candidate index out of range");
    return PSR_EINVAL;
  }
  const Confirmed &r = o->o.candidates[i];
  *out = r.s;
  if (profile_bins) std::copy(r.profile.values.begin(), r.profile.values.end(), profile_bins);
  if (profile_counts)
    std::copy(r.profile.counts.begin(), r.profile.counts.end(), profile_counts);
  return PSR_OK;
}

uint64_t psr_outcome_json(const psr_outcome *o, int pretty, char *buf, uint64_t len) {
  if (!o) return 0;
  const std::string s = psrjson::dump(outcome_json(o->o), pretty != 0);
  if (buf && len) {
    const uint64_t n = std::min<uint64_t>(len - 1, s.size());
    std::memcpy(buf, s.data(), n);
    buf[n] = '\0';
  }
  return s.size();
}

void psr_outcome_free(psr_outcome *o) { delete o; }

}  // extern "C"
