// ORACLE - TEST INFRASTRUCTURE ONLY (see psr_oracle.h for the parity status).
//
// Operation-by-operation CPU restatement of the PulsarSr search path.  Each
// function cites the reference lines it follows (paths inside the reference
// project).  Compile with -ffp-contract=off: Rust never contracts a*b+c.
#include "psr_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

namespace {

thread_local std::string g_err;

int fail(const std::string &msg) {
  g_err = msg;
  return 1;
}

const double K_DM = 4148.808;  // dedisperse/src/lib.rs:3

// ---------------------------------------------------------------- ordering
// Rust f32::total_cmp / f64::total_cmp as a strict-weak "less".
inline int32_t key32(float x) {
  int32_t i;
  std::memcpy(&i, &x, 4);
  return i ^ (int32_t)((uint32_t)(i >> 31) >> 1);
}
inline int64_t key64(double x) {
  int64_t i;
  std::memcpy(&i, &x, 8);
  return i ^ (int64_t)((uint64_t)(i >> 63) >> 1);
}
inline bool tless32(float a, float b) { return key32(a) < key32(b); }
inline int tcmp64(double a, double b) {
  int64_t x = key64(a), y = key64(b);
  return x < y ? -1 : (x > y ? 1 : 0);
}

// Rust `iter().sum::<f32>()`: sequential, no reassociation.
inline float seq_sum_f32(const float *v, size_t n) {
  float s = -0.0f;
  for (size_t i = 0; i < n; ++i) s += v[i];
  return s;
}

// ------------------------------------------------------------ rfi::median
// rfi/src/lib.rs:4-12: upper median v[len/2] after select_nth_unstable_by
// (total_cmp).  The selected VALUE is unique, whatever the selection method.
float median_f32(const float *values, size_t n) {
  if (n == 0) return 0.0f;
  std::vector<float> v(values, values + n);
  size_t i = n / 2;
  std::nth_element(v.begin(), v.begin() + i, v.end(), tless32);
  return v[i];
}

// rfi/src/lib.rs:13-22
std::vector<bool> outliers(const std::vector<float> &v, float threshold) {
  float center = median_f32(v.data(), v.size());
  std::vector<float> dev(v.size());
  for (size_t i = 0; i < v.size(); ++i) dev[i] = std::fabs(v[i] - center);
  float mad = median_f32(dev.data(), dev.size());
  float scale = std::fmax(std::fmax(1.4826f * mad, std::fabs(center) * 1e-4f),
                          1e-6f);
  std::vector<bool> out(v.size());
  for (size_t i = 0; i < v.size(); ++i)
    out[i] = std::fabs(v[i] - center) > threshold * scale;
  return out;
}

struct Mask {
  std::vector<uint64_t> channels, blocks;
  uint64_t block_samples = 0;
  double masked_fraction = 0;
};

// rfi/src/lib.rs:31-96
Mask rfi_mask(float *data, size_t nsamples, size_t nchans, size_t block_samples,
              float threshold) {
  std::vector<float> means(nchans), variances(nchans);
  for (size_t c = 0; c < nchans; ++c)
    means[c] = seq_sum_f32(data + c * nsamples, nsamples) / (float)nsamples;
  for (size_t c = 0; c < nchans; ++c) {
    const float *row = data + c * nsamples;
    float m = means[c];
    float s = -0.0f;
    for (size_t t = 0; t < nsamples; ++t) {
      float d = row[t] - m;
      s += d * d;
    }
    variances[c] = s / (float)nsamples;
  }
  std::vector<bool> means_bad = outliers(means, threshold);
  std::vector<bool> vars_bad = outliers(variances, threshold);
  Mask m;
  std::vector<bool> bad(nchans, false);
  for (size_t c = 0; c < nchans; ++c)
    if (means_bad[c] || vars_bad[c] || variances[c] < 1e-12f) {
      m.channels.push_back(c);
      bad[c] = true;
    }
  size_t blocks_n = (nsamples + block_samples - 1) / block_samples;
  size_t active = nchans - m.channels.size();
  std::vector<float> block_means(blocks_n);
  for (size_t b = 0; b < blocks_n; ++b) {
    size_t start = b * block_samples;
    size_t end = std::min(start + block_samples, nsamples);
    float sum = 0.0f;
    for (size_t c = 0; c < nchans; ++c)
      if (!bad[c]) sum += seq_sum_f32(data + c * nsamples + start, end - start);
    block_means[b] = sum / (float)((end - start) * std::max<size_t>(active, 1));
  }
  std::vector<bool> bo = outliers(block_means, threshold);
  for (size_t b = 0; b < blocks_n; ++b)
    if (bo[b]) m.blocks.push_back(b);
  size_t count = m.channels.size() * nsamples;
  for (size_t c = 0; c < nchans; ++c) {
    float *row = data + c * nsamples;
    float typical = median_f32(row, nsamples);
    if (bad[c]) {
      std::fill(row, row + nsamples, typical);
    } else {
      for (uint64_t b : m.blocks) {
        size_t start = b * block_samples;
        size_t end = std::min(start + block_samples, nsamples);
        std::fill(row + start, row + end, typical);
        count += end - start;
      }
    }
  }
  m.block_samples = block_samples;
  m.masked_fraction = (double)count / (double)(nchans * nsamples);
  return m;
}

// ------------------------------------------------------------ dedisperse
// dedisperse/src/lib.rs:9-34.  f.powi(-2) is 1/(f*f).
bool delays(const double *f, size_t n, double tsamp, double dm,
            std::vector<uint64_t> &out) {
  bool bad = n == 0 || !std::isfinite(tsamp) || tsamp <= 0.0 ||
             !std::isfinite(dm) || dm < 0.0;
  for (size_t i = 0; i < n && !bad; ++i)
    if (!std::isfinite(f[i]) || f[i] <= 0.0) bad = true;
  if (bad) {
    g_err =
        "invalid dedispersion input: positive frequencies/tsamp and "
        "nonnegative DM required";
    return false;
  }
  double reference = 0.0;
  for (size_t i = 0; i < n; ++i) reference = std::fmax(reference, f[i]);
  double rinv = 1.0 / (reference * reference);
  out.resize(n);
  for (size_t i = 0; i < n; ++i) {
    double finv = 1.0 / (f[i] * f[i]);
    double samples = std::round(K_DM * dm * (finv - rinv) / tsamp);
    if (samples > 18446744073709551615.0) {
      g_err = "invalid dedispersion input: delay overflow";
      return false;
    }
    out[i] = samples > 0.0 ? (uint64_t)samples : 0;
  }
  return true;
}

// dedisperse/src/lib.rs:35-44
bool dm_step(const double *f, size_t n, double tsamp, double &out) {
  std::vector<uint64_t> tmp;
  if (!delays(f, n, tsamp, 0.0, tmp)) return false;
  double lo = INFINITY, hi = 0.0;
  for (size_t i = 0; i < n; ++i) {
    lo = std::fmin(lo, f[i]);
    hi = std::fmax(hi, f[i]);
  }
  double span = K_DM * (1.0 / (lo * lo) - 1.0 / (hi * hi));
  if (span <= 0.0) {
    g_err = "invalid dedispersion input: DM planning requires finite bandwidth";
    return false;
  }
  out = tsamp / span;
  return true;
}

// dedisperse/src/lib.rs:45-60
bool plan(double mn, double mx, double step, std::vector<double> &out) {
  if (!std::isfinite(mn) || !std::isfinite(mx) || !std::isfinite(step) ||
      mn < 0.0 || mx < mn || step <= 0.0) {
    g_err = "invalid dedispersion input: invalid DM bounds/step";
    return false;
  }
  double nf = std::floor((mx - mn) / step);
  size_t n = (size_t)nf + 1;
  if (n > 100000) {
    g_err = "invalid dedispersion input: more than 100000 DM trials";
    return false;
  }
  out.resize(n);
  for (size_t i = 0; i < n; ++i) out[i] = mn + (double)i * step;
  return true;
}

// dedisperse/src/lib.rs:61-90: channel-order f32 accumulation.
bool apply(const float *data, size_t nchans, size_t nsamples,
           const uint64_t *d, int64_t length, std::vector<float> &out) {
  if (nchans == 0 || nsamples == 0) {
    g_err = "invalid dedispersion input: array shape mismatch";
    return false;
  }
  uint64_t max_delay = 0;
  for (size_t c = 0; c < nchans; ++c) max_delay = std::max(max_delay, d[c]);
  if (max_delay > nsamples) {
    g_err = "invalid dedispersion input: delay exceeds observation";
    return false;
  }
  size_t available = nsamples - max_delay;
  size_t n = length < 0 ? available : (size_t)length;
  if (n < 2 || n > available) {
    g_err = "invalid dedispersion input: invalid output length";
    return false;
  }
  out.assign(n, 0.0f);
  for (size_t c = 0; c < nchans; ++c) {
    const float *row = data + c * nsamples + d[c];
    for (size_t t = 0; t < n; ++t) out[t] += row[t];
  }
  return true;
}

// ------------------------------------------------------------------ FFT
// The oracle's FP32 real FFT.  Definition (the CUDA path reproduces it):
//   N = 2*next_pow2(len) real points, M = N/2 complex points.
//   z[n] = x[2n] + i x[2n+1], x[i] = series[i] - (f32)mean for i < len, else 0.
//   Twiddles W_N^x = exp(-2 pi i x / N) from a quarter table Q[r] =
//   ((f32)cos(2 pi r/N), (f32)sin(2 pi r/N)) for r <= N/8, mirrored
//   Q[r] = (Q[N/4-r].sin, Q[N/4-r].cos) for N/8 < r <= N/4, then quadrant
//   symmetry (exact).  cmul(a,w) = (fmaf(a.re,w.re,-(a.im*w.im)),
//   fmaf(a.re,w.im,a.im*w.re)); every other operation is a plain f32 op.
//   Complex FFT of size M: M <= 4096 -> one Stockham sub-FFT; otherwise
//   four-step M = M1*M2 (M1 = 2^ceil(m/2)): column sub-FFTs of size M1 over
//   n1 (n = n1*M2 + n2), twiddle W_M^(n2*k1), row sub-FFTs of size M2,
//   Z[k1 + M1*k2].  Sub-FFT of size L: Stockham autosort stages with radices
//   [16]*(q/4) + [2,4,8][q%4-1]; DFT_8 and DFT_16 are four-step 2x4 and 4x4
//   built from DFT_2/DFT_4 with the internal twiddles W_R^(n2*k1).
//   Real post-processing for k in [0, M]:
//     a = Z[k%M], b = conj(Z[(M-k)%M]), e = a+b, o = a-b, t = cmul(o, W_N^k),
//     X = (0.5*(e.re + t.im), 0.5*(e.im - t.re)), power = X.re^2 + X.im^2.
struct cf {
  float re, im;
};
inline cf cadd(cf a, cf b) { return {a.re + b.re, a.im + b.im}; }
inline cf csub(cf a, cf b) { return {a.re - b.re, a.im - b.im}; }
inline cf cmulw(cf a, cf w) {
  return {std::fmaf(a.re, w.re, -(a.im * w.im)),
          std::fmaf(a.re, w.im, a.im * w.re)};
}
inline cf mul_mi(cf d) { return {d.im, -d.re}; }

struct Twiddle {
  size_t N;
  std::vector<cf> Q;
  explicit Twiddle(size_t n) : N(n), Q(n / 4 + 1) {
    size_t n8 = n / 8, n4 = n / 4;
    for (size_t r = 0; r <= n8; ++r) {
      double a = 6.283185307179586 * (double)r / (double)n;
      Q[r] = {(float)std::cos(a), (float)std::sin(a)};
    }
    for (size_t r = n8 + 1; r <= n4; ++r) Q[r] = {Q[n4 - r].im, Q[n4 - r].re};
  }
  cf w(size_t x) const {
    size_t q4 = N / 4, q = x / q4, r = x % q4;
    float c = Q[r].re, s = Q[r].im;
    switch (q) {
      case 0: return {c, -s};
      case 1: return {-s, -c};
      case 2: return {-c, s};
      default: return {s, c};
    }
  }
};

void dft2(cf *v) {
  cf a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}
void dft4(cf *v) {
  cf a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
  cf c = cadd(v[1], v[3]), d = mul_mi(csub(v[1], v[3]));
  v[0] = cadd(a, c);
  v[1] = cadd(b, d);
  v[2] = csub(a, c);
  v[3] = csub(b, d);
}
// DFT_R, R = A*B: n = n1*B + n2, k = k1 + A*k2.
void dft_ab(cf *v, int A, int B, const Twiddle &T) {
  int R = A * B;
  cf u[16][16];
  cf tmp[16];
  for (int n2 = 0; n2 < B; ++n2) {
    for (int n1 = 0; n1 < A; ++n1) tmp[n1] = v[n1 * B + n2];
    if (A == 2) dft2(tmp); else dft4(tmp);
    for (int k1 = 0; k1 < A; ++k1) u[n2][k1] = tmp[k1];
  }
  for (int n2 = 1; n2 < B; ++n2)
    for (int k1 = 1; k1 < A; ++k1)
      u[n2][k1] = cmulw(u[n2][k1], T.w((size_t)(n2 * k1) * (T.N / R)));
  for (int k1 = 0; k1 < A; ++k1) {
    for (int n2 = 0; n2 < B; ++n2) tmp[n2] = u[n2][k1];
    if (B == 2) dft2(tmp); else dft4(tmp);
    for (int k2 = 0; k2 < B; ++k2) v[k1 + A * k2] = tmp[k2];
  }
}
void dftR(cf *v, int R, const Twiddle &T) {
  switch (R) {
    case 2: dft2(v); break;
    case 4: dft4(v); break;
    case 8: dft_ab(v, 2, 4, T); break;
    default: dft_ab(v, 4, 4, T); break;
  }
}
std::vector<int> radix_list(size_t L) {
  int q = 0;
  while (((size_t)1 << q) < L) ++q;
  std::vector<int> r(q / 4, 16);
  if (q % 4) r.push_back(q % 4 == 1 ? 2 : (q % 4 == 2 ? 4 : 8));
  return r;
}
// Stockham autosort sub-FFT of length L (power of two) in place.
void subfft(cf *x, size_t L, const Twiddle &T, std::vector<cf> &scratch) {
  if (L == 1) return;
  scratch.resize(L);
  cf *src = x, *dst = scratch.data();
  size_t Ns = 1;
  for (int R : radix_list(L)) {
    size_t stride = L / R;
    for (size_t j = 0; j < stride; ++j) {
      size_t k = j % Ns;
      cf v[16];
      for (int r = 0; r < R; ++r) v[r] = src[j + r * stride];
      if (Ns > 1 && k != 0)
        for (int r = 1; r < R; ++r)
          v[r] = cmulw(v[r], T.w((size_t)r * k * (T.N / (Ns * R))));
      dftR(v, R, T);
      size_t base = (j / Ns) * Ns * R + k;
      for (int r = 0; r < R; ++r) dst[base + r * Ns] = v[r];
    }
    std::swap(src, dst);
    Ns *= R;
  }
  if (src != x) std::copy(src, src + L, x);
}

void complex_fft(std::vector<cf> &z, const Twiddle &T) {
  size_t M = z.size();
  int m = 0;
  while (((size_t)1 << m) < M) ++m;
  std::vector<cf> scratch;
  if (m <= 12) {
    subfft(z.data(), M, T, scratch);
    return;
  }
  size_t M1 = (size_t)1 << ((m + 1) / 2), M2 = (size_t)1 << (m / 2);
  std::vector<cf> Y(M), col(M1), row(M2);
  for (size_t n2 = 0; n2 < M2; ++n2) {
    for (size_t n1 = 0; n1 < M1; ++n1) col[n1] = z[n1 * M2 + n2];
    subfft(col.data(), M1, T, scratch);
    for (size_t k1 = 0; k1 < M1; ++k1) {
      cf v = col[k1];
      if (n2 * k1 != 0) v = cmulw(v, T.w(2 * n2 * k1));
      Y[k1 * M2 + n2] = v;
    }
  }
  for (size_t k1 = 0; k1 < M1; ++k1) {
    for (size_t n2 = 0; n2 < M2; ++n2) row[n2] = Y[k1 * M2 + n2];
    subfft(row.data(), M2, T, scratch);
    for (size_t k2 = 0; k2 < M2; ++k2) z[k1 + M1 * k2] = row[k2];
  }
}

size_t next_pow2(size_t n) {
  size_t p = 1;
  while (p < n) p <<= 1;
  return p;
}

// search/src/lib.rs:35-44: mean (f64), subtract as f32, real FFT, norm_sqr.
std::vector<float> raw_power(const float *series, size_t len) {
  size_t N = next_pow2(len) * 2, M = N / 2;
  double mean = -0.0;
  for (size_t i = 0; i < len; ++i) mean += (double)series[i];
  mean /= (double)len;
  float mf = (float)mean;
  std::vector<cf> z(M, cf{0.0f, 0.0f});
  for (size_t i = 0; i < len; ++i) {
    float v = series[i] - mf;
    if (i & 1) z[i >> 1].im = v; else z[i >> 1].re = v;
  }
  Twiddle T(N);
  complex_fft(z, T);
  std::vector<float> p(M + 1);
  for (size_t k = 0; k <= M; ++k) {
    cf a = z[k % M], bz = z[(M - k) % M];
    cf b = {bz.re, -bz.im};
    cf e = cadd(a, b), o = csub(a, b);
    cf t = cmulw(o, T.w(k));
    float xr = 0.5f * (e.re + t.im), xi = 0.5f * (e.im - t.re);
    p[k] = xr * xr + xi * xi;
  }
  return p;
}

// FP64 reference: iterative radix-2 complex FFT of the same real input.
std::vector<double> raw_power_f64(const float *series, size_t len) {
  size_t N = next_pow2(len) * 2;
  double mean = -0.0;
  for (size_t i = 0; i < len; ++i) mean += (double)series[i];
  mean /= (double)len;
  float mf = (float)mean;
  std::vector<double> re(N, 0.0), im(N, 0.0);
  for (size_t i = 0; i < len; ++i) re[i] = (double)(series[i] - mf);
  for (size_t i = 1, j = 0; i < N; ++i) {
    size_t bit = N >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(re[i], re[j]);
  }
  for (size_t len2 = 2; len2 <= N; len2 <<= 1) {
    double ang = -6.283185307179586476925 / (double)len2;
    for (size_t i = 0; i < N; i += len2)
      for (size_t k = 0; k < len2 / 2; ++k) {
        double wr = std::cos(ang * (double)k), wi = std::sin(ang * (double)k);
        size_t a = i + k, b = i + k + len2 / 2;
        double xr = re[b] * wr - im[b] * wi, xi = re[b] * wi + im[b] * wr;
        re[b] = re[a] - xr;
        im[b] = im[a] - xi;
        re[a] += xr;
        im[a] += xi;
      }
  }
  std::vector<double> p(N / 2 + 1);
  for (size_t k = 0; k <= N / 2; ++k) p[k] = re[k] * re[k] + im[k] * im[k];
  return p;
}

// --------------------------------------------------------- periodicity
struct Cand {
  double frequency_hz, period_s, dm;
  uint64_t harmonics;
  double score;
};
struct Config {
  double min_hz = 1, max_hz = INFINITY, threshold = 6;
  size_t max_candidates = 32;
  std::vector<std::pair<double, double>> birdies;
  size_t max_harmonics = 16;  // 32 extends the reference's level list by h = 32
};

void stable_sort_by_score_desc(std::vector<Cand> &c) {
  std::stable_sort(c.begin(), c.end(), [](const Cand &a, const Cand &b) {
    return tcmp64(b.score, a.score) < 0;
  });
}

// search/src/lib.rs:33-145
std::vector<Cand> periodicity(const float *series, size_t len, double tsamp,
                              double dm, const Config &cfg) {
  std::vector<float> raw = raw_power(series, len);
  size_t plen = raw.size();
  size_t size = (plen - 1) * 2;
  double fsum = -0.0;
  for (float p : raw) fsum += (double)p;
  float floor_ = (float)(fsum / (double)plen * 1e-6);
  std::vector<float> power(plen);
  for (size_t b = 0; b * 64 < plen; ++b) {
    size_t center = b * 64;
    size_t lo = std::max<size_t>(center >= 128 ? center - 128 : 0, 1);
    size_t hi = std::min(center + 192, plen);
    float scale = std::fmax(
        std::fmax(median_f32(raw.data() + lo, hi - lo) / 0.693147180559945309f,
                  floor_),
        1e-20f);
    for (size_t i = center; i < std::min(center + 64, plen); ++i)
      power[i] = raw[i] / scale;
  }
  power[0] = 0.0f;
  double bin_hz = 1.0 / ((double)size * tsamp);
  for (size_t i = 0; i < plen; ++i) {
    double f = (double)i * bin_hz;
    for (auto &bd : cfg.birdies)
      if (std::fabs(f - bd.first) <= bd.second) {
        power[i] = 0.0f;
        break;
      }
  }
  size_t first = (size_t)std::fmax(std::ceil(cfg.min_hz / bin_hz), 1.0);
  double lastf = std::floor(std::fmin(cfg.max_hz, 0.5 / tsamp) / bin_hz);
  size_t last = std::min(lastf <= 0 ? (size_t)0 : (size_t)lastf, plen - 2);
  auto offset_at = [&](size_t k) {
    double curvature =
        (double)raw[k - 1] - 2.0 * (double)raw[k] + (double)raw[k + 1];
    if (curvature < 0.0) {
      double o = 0.5 * ((double)raw[k - 1] - (double)raw[k + 1]) / curvature;
      return std::fmin(std::fmax(o, -0.5), 0.5);
    }
    return 0.0;
  };
  std::vector<Cand> cands;
  for (size_t h : {1, 2, 4, 8, 16, 32}) {
    if (h > cfg.max_harmonics) break;
    size_t end = std::min(last, (plen - 2) / h);
    if (end <= first + 1) continue;
    std::vector<double> scores(end - first + 1);
    for (size_t k = first; k <= end; ++k) {
      if (h > 1 && power[k] < 4.0f) {
        scores[k - first] = -INFINITY;
        continue;
      }
      double off = offset_at(k);
      double sum = -0.0;
      for (size_t j = 1; j <= h; ++j) {
        double position = ((double)k + off) * (double)j;
        size_t index = (size_t)std::round(position);
        sum += (double)power[std::min(index, plen - 1)];
      }
      scores[k - first] = (sum - (double)h) / std::sqrt((double)h);
    }
    for (size_t i = 1; i + 1 < scores.size(); ++i) {
      if (scores[i] >= cfg.threshold && scores[i] > scores[i - 1] &&
          scores[i] >= scores[i + 1]) {
        size_t k = first + i;
        double f = ((double)k + offset_at(k)) * bin_hz;
        cands.push_back({f, 1.0 / f, dm, h, scores[i]});
      }
    }
  }
  stable_sort_by_score_desc(cands);
  std::vector<Cand> kept;
  double tol = 1.0 / ((double)len * tsamp);
  for (const Cand &c : cands) {
    bool dup = false;
    for (const Cand &k : kept)
      if (std::fabs(k.frequency_hz - c.frequency_hz) < tol) {
        dup = true;
        break;
      }
    if (dup) continue;
    kept.push_back(c);
    if (kept.size() >= cfg.max_candidates) break;
  }
  return kept;
}

// search/src/lib.rs:147-176
std::vector<Cand> sift(std::vector<Cand> c, double res, size_t limit,
                       bool reject_dm_zero) {
  stable_sort_by_score_desc(c);
  std::vector<Cand> kept;
  std::vector<double> rejected;
  for (const Cand &x : c) {
    auto related = [&](double f) {
      for (int h = 1; h <= 16; ++h)
        if (std::fabs(x.frequency_hz - f * h) <= res ||
            std::fabs(f - x.frequency_hz * h) <= res)
          return true;
      return false;
    };
    bool skip = false;
    for (auto &k : kept) skip = skip || related(k.frequency_hz);
    for (double f : rejected) skip = skip || related(f);
    if (skip) continue;
    if (reject_dm_zero && x.dm <= 0.0) {
      rejected.push_back(x.frequency_hz);
      continue;
    }
    kept.push_back(x);
    if (kept.size() >= limit) break;
  }
  return kept;
}

// --------------------------------------------------------------- fold
struct Profile {
  double period_s = 0, snr = 0, rcs = 0;
  std::vector<float> bins;
  std::vector<uint64_t> counts;
};

// fold/src/lib.rs:16-80
Profile profile_at(const float *series, size_t n, double tsamp, double period,
                   size_t bins, size_t offset) {
  std::vector<double> sums(bins, 0.0);
  std::vector<uint64_t> counts(bins, 0);
  for (size_t t = 0; t < n; ++t) {
    double x = (double)(t + offset) * tsamp / period;
    double phase = x - std::trunc(x);
    size_t b = std::min((size_t)(phase * (double)bins), bins - 1);
    sums[b] += (double)series[t];
    counts[b] += 1;
  }
  Profile p;
  p.period_s = period;
  p.bins.resize(bins);
  for (size_t b = 0; b < bins; ++b)
    p.bins[b] = counts[b] > 0 ? (float)(sums[b] / (double)counts[b]) : 0.0f;
  float center = median_f32(p.bins.data(), bins);
  std::vector<float> off;
  for (size_t b = 0; b < bins; ++b)
    if (counts[b] > 0) off.push_back(p.bins[b]);
  std::sort(off.begin(), off.end(), tless32);
  off.resize(std::max<size_t>(off.size() * 3 / 4, 1));
  double mean = -0.0;
  for (float v : off) mean += (double)v;
  mean /= (double)off.size();
  double var = -0.0;
  for (float v : off) {
    double d = (double)v - mean;
    var += d * d;
  }
  double sigma = std::sqrt(var / (double)off.size());
  float peak = -INFINITY;
  for (float v : p.bins) peak = std::fmax(peak, v);
  p.snr = sigma > 1e-12 ? ((double)peak - (double)center) / sigma : 0.0;
  double smean = -0.0;
  for (size_t t = 0; t < n; ++t) smean += (double)series[t];
  smean /= (double)n;
  double svar = -0.0;
  for (size_t t = 0; t < n; ++t) {
    double d = (double)series[t] - smean;
    svar += d * d;
  }
  svar /= (double)n;
  size_t populated = 0;
  for (auto c : counts) populated += c > 0;
  if (svar > 1e-12 && populated > 1) {
    double s = -0.0;
    for (size_t b = 0; b < bins; ++b) {
      double d = (double)p.bins[b] - smean;
      s += (double)counts[b] * (d * d) / svar;
    }
    p.rcs = s / (double)(populated - 1);
  } else {
    p.rcs = 0.0;
  }
  p.counts = counts;
  return p;
}

// fold/src/lib.rs:81-97 (max_by keeps the LAST maximum).
Profile refine(const float *series, size_t n, double tsamp, double frequency,
               double span, size_t steps, size_t bins) {
  Profile best;
  bool have = false;
  for (size_t i = 0; i <= steps; ++i) {
    double f = frequency - span + 2.0 * span * (double)i / (double)steps;
    Profile p = profile_at(series, n, tsamp, 1.0 / f, bins, 0);
    if (!have || tcmp64(p.rcs, best.rcs) >= 0) {
      best = std::move(p);
      have = true;
    }
  }
  return best;
}

// ------------------------------------------------------- confirmation
struct Window {
  size_t start_bin, width_bins, bins;
  bool contains(size_t b) const {
    return (b + bins - start_bin) % bins < width_bins;
  }
};
struct Measurement {
  double snr;
  size_t on, off;
  double diff, err;
};

// confirmation.rs:103-105
inline size_t phase_bin(size_t t, double tsamp, double period, size_t bins) {
  double x = (double)t * tsamp / period;
  return std::min((size_t)((x - std::trunc(x)) * (double)bins), bins - 1);
}

// confirmation.rs:107-141
Measurement measure(const float *x, size_t n, size_t offset, double tsamp,
                    double period, const Window &w) {
  size_t cnt[2] = {0, 0};
  double sum[2] = {-0.0, -0.0}, sum2[2] = {-0.0, -0.0};
  for (size_t i = 0; i < n; ++i) {
    int k = w.contains(phase_bin(i + offset, tsamp, period, w.bins)) ? 1 : 0;
    double v = (double)x[i];
    cnt[k] += 1;
    sum[k] += v;
    sum2[k] += v * v;
  }
  if (cnt[0] < 2 || cnt[1] < 2) return {0.0, cnt[1], cnt[0], 0.0, 0.0};
  double difference = sum[1] / (double)cnt[1] - sum[0] / (double)cnt[0];
  auto variance = [&](int k) {
    return std::fmax(
        (sum2[k] - sum[k] * sum[k] / (double)cnt[k]) / (double)(cnt[k] - 1),
        0.0);
  };
  double error =
      std::sqrt(variance(1) / (double)cnt[1] + variance(0) / (double)cnt[0]);
  return {error > 1e-10 ? difference / error : 0.0, cnt[1], cnt[0], difference,
          error};
}

// confirmation.rs:142-176
Window select_window(const Profile &p) {
  size_t bins = p.bins.size();
  double best = -INFINITY;
  Window w{0, 1, bins};
  for (size_t width = 1; width <= bins / 4; width <<= 1) {
    for (size_t start = 0; start < bins; ++start) {
      double on = -0.0;
      for (size_t j = 0; j < width; ++j) on += (double)p.bins[(start + j) % bins];
      double total = -0.0;
      for (float v : p.bins) total += (double)v;
      double contrast = on / (double)width - (total - on) / (double)(bins - width);
      double score =
          contrast / std::sqrt(1.0 / (double)width + 1.0 / (double)(bins - width));
      if (score > best) {
        best = score;
        w = {start, width, bins};
      }
    }
  }
  return w;
}

struct Family {
  Cand leader;
  std::vector<Cand> members;
};

// confirmation.rs:177-199
std::vector<Family> group(const std::vector<Cand> &cands, double res,
                          size_t limit) {
  std::vector<Cand> sorted = cands;
  stable_sort_by_score_desc(sorted);
  std::vector<Family> fam;
  for (const Cand &c : sorted) {
    Family *hit = nullptr;
    for (auto &f : fam) {
      const Cand &a = f.leader;
      bool rel = false;
      for (int h = 1; h <= 16 && !rel; ++h)
        rel = std::fabs(a.frequency_hz - c.frequency_hz * h) <= res ||
              std::fabs(c.frequency_hz - a.frequency_hz * h) <= res;
      if (rel) {
        hit = &f;
        break;
      }
    }
    if (hit) hit->members.push_back(c);
    else if (fam.size() < limit) fam.push_back({c, {c}});
  }
  return fam;
}

// ------------------------------------------------------------- JSON
struct Json {
  std::string s;
  void raw(const std::string &x) { s += x; }
  void f64(double v) {
    if (!std::isfinite(v)) {
      s += "null";
      return;
    }
    char b[40];
    std::snprintf(b, sizeof b, "%.17g", v);
    s += b;
  }
  void f32(float v) {
    if (!std::isfinite(v)) {
      s += "null";
      return;
    }
    char b[40];
    std::snprintf(b, sizeof b, "%.9g", (double)v);
    s += b;
  }
  void u64(uint64_t v) { s += std::to_string(v); }
  void key(const char *k) {
    s += '"';
    s += k;
    s += "\":";
  }
};

void json_cand(Json &j, const Cand &c) {
  j.raw("{");
  j.key("frequency_hz"); j.f64(c.frequency_hz); j.raw(",");
  j.key("period_s"); j.f64(c.period_s); j.raw(",");
  j.key("dm"); j.f64(c.dm); j.raw(",");
  j.key("harmonics"); j.u64(c.harmonics); j.raw(",");
  j.key("score"); j.f64(c.score);
  j.raw("}");
}
void json_profile(Json &j, const Profile &p) {
  j.raw("{");
  j.key("period_s"); j.f64(p.period_s); j.raw(",");
  j.key("snr"); j.f64(p.snr); j.raw(",");
  j.key("reduced_chi_square"); j.f64(p.rcs); j.raw(",");
  j.key("bins"); j.raw("[");
  for (size_t i = 0; i < p.bins.size(); ++i) { if (i) j.raw(","); j.f32(p.bins[i]); }
  j.raw("],");
  j.key("counts"); j.raw("[");
  for (size_t i = 0; i < p.counts.size(); ++i) { if (i) j.raw(","); j.u64(p.counts[i]); }
  j.raw("]}");
}
void json_meas(Json &j, const Measurement &m) {
  j.raw("{");
  j.key("snr"); j.f64(m.snr); j.raw(",");
  j.key("on_samples"); j.u64(m.on); j.raw(",");
  j.key("off_samples"); j.u64(m.off); j.raw(",");
  j.key("mean_difference"); j.f64(m.diff); j.raw(",");
  j.key("standard_error"); j.f64(m.err);
  j.raw("}");
}
void json_window(Json &j, const Window &w) {
  j.raw("{");
  j.key("start_bin"); j.u64(w.start_bin); j.raw(",");
  j.key("width_bins"); j.u64(w.width_bins); j.raw(",");
  j.key("bins"); j.u64(w.bins);
  j.raw("}");
}

// Periodicity of every trial (the psr search loop, cli/src/main.rs:462-473):
// worker threads over trials, concatenated in trial order.
std::vector<std::vector<Cand>> search_trials(
    const float *data, size_t nchans, size_t nsamples, const double *freqs,
    double tsamp, const double *trials, size_t ntrials, size_t discovery,
    const Config &cfg, int threads, std::string &err) {
  std::vector<std::vector<Cand>> lists(ntrials);
  std::vector<std::string> errs(ntrials);
  std::atomic<size_t> next{0};
  auto work = [&]() {
    std::vector<uint64_t> d;
    std::vector<float> x;
    for (;;) {
      size_t i = next.fetch_add(1);
      if (i >= ntrials) return;
      if (!delays(freqs, nchans, tsamp, trials[i], d) ||
          !apply(data, nchans, nsamples, d.data(), (int64_t)discovery, x)) {
        errs[i] = g_err;
        continue;
      }
      lists[i] = periodicity(x.data(), x.size(), tsamp, trials[i], cfg);
    }
  };
  int nt = std::max(threads, 1);
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(work);
  work();
  for (auto &t : pool) t.join();
  for (auto &e : errs)
    if (!e.empty()) {
      err = e;
      break;
    }
  return lists;
}

// confirmation.rs:203-496, serialised as the schema-2 Outcome.
bool analyze(const float *data, size_t nsamples, const std::vector<double> &freqs,
             double tsamp, const std::vector<double> &trials,
             const std::vector<Cand> &generated, size_t limit, size_t bins,
             Json &j) {
  size_t nch = freqs.size();
  if (trials.empty() || limit == 0 || bins < 8 || nch < 4) {
    g_err =
        "invalid dedispersion input: confirmation requires >=4 channels, >=8 "
        "bins and valid array/trials";
    return false;
  }
  for (size_t i = 1; i < trials.size(); ++i)
    if (trials[i] <= trials[i - 1]) {
      g_err = "invalid dedispersion input: DM trials must increase";
      return false;
    }
  double max_dm = trials.back();
  std::vector<uint64_t> dmax;
  if (!delays(freqs.data(), nch, tsamp, max_dm, dmax)) return false;
  uint64_t guard = *std::max_element(dmax.begin(), dmax.end());
  if (guard > nsamples || nsamples - guard < 512) {
    g_err = "invalid dedispersion input: observation too short for confirmation";
    return false;
  }
  size_t length = nsamples - guard;
  if (guard > length || length - guard < 256) {
    g_err = "invalid dedispersion input: DM delay leaves no independent split";
    return false;
  }
  size_t discovery = (length - guard) / 2;
  size_t vstart = discovery + guard;
  size_t validation = length - vstart;
  double resolution = 1.0 / ((double)discovery * tsamp);
  double step = trials.size() > 1 ? trials[1] - trials[0] : 1.0;
  std::vector<uint64_t> zeros(nch, 0);
  std::vector<float> zero_series, x;
  if (!apply(data, nch, nsamples, zeros.data(), (int64_t)discovery, zero_series))
    return false;
  Config zc;
  zc.min_hz = 1.0;
  zc.max_hz = 0.5 / tsamp;
  zc.threshold = 8.0;
  zc.max_candidates = 64;
  std::vector<Cand> zero_c =
      periodicity(zero_series.data(), zero_series.size(), tsamp, 0.0, zc);

  j.raw("{");
  j.key("rules");
  j.raw("{\"version\":\"split-confirm-v1\",\"minimum_validation_snr\":6.0,"
        "\"minimum_part_snr\":1.0,\"minimum_time_parts\":3,"
        "\"minimum_subbands\":3,\"minimum_dm_contrast\":1.25,"
        "\"minimum_dispersion_widths\":1.5,"
        "\"maximum_zero_dm_spectral_ratio\":1.0},");
  j.key("discovery_samples"); j.u64(discovery); j.raw(",");
  j.key("validation_start_sample"); j.u64(vstart); j.raw(",");
  j.key("validation_samples"); j.u64(validation); j.raw(",");
  j.key("common_samples"); j.u64(length); j.raw(",");
  j.key("trial_count"); j.u64(trials.size()); j.raw(",");
  j.key("candidates"); j.raw("[");
  std::vector<Family> fams = group(generated, resolution * 1.5, limit);
  for (size_t fi = 0; fi < fams.size(); ++fi) {
    const Cand &cand = fams[fi].leader;
    const std::vector<Cand> &members = fams[fi].members;
    double zero_ratio = 0.0;
    for (const Cand &z : zero_c) {
      bool rel = false;
      for (int m = 1; m <= 16 && !rel; ++m)
        for (int n = 1; n <= 16 && !rel; ++n)
          rel = std::fabs(cand.frequency_hz -
                          z.frequency_hz * (double)m / (double)n) <=
                resolution * 1.5;
      if (rel) zero_ratio = std::fmax(zero_ratio, z.score / std::fmax(cand.score, 1.0));
    }
    std::vector<uint64_t> d;
    if (!delays(freqs.data(), nch, tsamp, cand.dm, d)) return false;
    std::vector<float> initial;
    if (!apply(data, nch, nsamples, d.data(), (int64_t)length, initial)) return false;
    Profile best =
        refine(initial.data(), discovery, tsamp, cand.frequency_hz, resolution, 40, bins);
    double best_dm = cand.dm;
    double period = best.period_s;
    for (int i = -10; i <= 10; ++i) {
      double dm = std::fmin(std::fmax(cand.dm + (double)i * step / 2.0, trials[0]), max_dm);
      if (!delays(freqs.data(), nch, tsamp, dm, d)) return false;
      if (!apply(data, nch, nsamples, d.data(), (int64_t)discovery, x)) return false;
      Profile p = profile_at(x.data(), x.size(), tsamp, period, bins, 0);
      if (p.rcs > best.rcs) {
        best = std::move(p);
        best_dm = dm;
      }
    }
    Window window = select_window(best);
    if (!delays(freqs.data(), nch, tsamp, best_dm, d)) return false;
    std::vector<float> series, zero;
    if (!apply(data, nch, nsamples, d.data(), (int64_t)length, series)) return false;
    Measurement vm = measure(series.data() + vstart, length - vstart, vstart, tsamp,
                             period, window);
    if (!apply(data, nch, nsamples, zeros.data(), (int64_t)length, zero)) return false;
    Profile zr = refine(zero.data() + vstart, length - vstart, tsamp, 1.0 / period,
                        resolution * 2.0, 40, bins);
    double zero_period = zr.period_s;
    Profile zp = profile_at(zero.data() + vstart, length - vstart, tsamp, zero_period,
                            bins, vstart);
    Window zw = select_window(zp);
    Measurement zm = measure(zero.data() + vstart, length - vstart, vstart, tsamp,
                             zero_period, zw);
    double contrast = std::fmax(vm.snr, 0.0) / std::fmax(zm.snr, 1.0);
    double dispersion_widths =
        ((double)*std::max_element(d.begin(), d.end()) * tsamp) /
        (period * (double)window.width_bins / (double)bins);
    std::vector<Measurement> parts, subs;
    std::vector<Profile> tprof, sprof;
    for (size_t part = 0; part < 4; ++part) {
      size_t lo = vstart + part * validation / 4;
      size_t hi = vstart + (part + 1) * validation / 4;
      parts.push_back(measure(series.data() + lo, hi - lo, lo, tsamp, period, window));
      tprof.push_back(profile_at(series.data() + lo, hi - lo, tsamp, period, bins, lo));
    }
    for (size_t part = 0; part < 4; ++part) {
      size_t lo = part * nch / 4, hi = (part + 1) * nch / 4;
      std::vector<float> sx;
      if (!apply(data + lo * nsamples, hi - lo, nsamples, d.data() + lo,
                 (int64_t)length, sx))
        return false;
      subs.push_back(measure(sx.data() + vstart, length - vstart, vstart, tsamp,
                             period, window));
      sprof.push_back(profile_at(sx.data() + vstart, length - vstart, tsamp, period,
                                 bins, vstart));
    }
    std::vector<std::vector<float>> chp(nch);
    for (size_t c = 0; c < nch; ++c)
      chp[c] = profile_at(data + c * nsamples, discovery, tsamp, period, bins, 0).bins;
    // DM response, confirmation.rs:397-433
    std::string resp;
    {
      Json r;
      r.raw("[");
      for (size_t ti = 0; ti < trials.size(); ++ti) {
        double dm = trials[ti];
        std::vector<uint64_t> dd;
        if (!delays(freqs.data(), nch, tsamp, dm, dd)) return false;
        std::vector<double> comb(bins, 0.0);
        for (size_t c = 0; c < nch; ++c) {
          const std::vector<float> &pr = chp[c];
          double mean = -0.0;
          for (float v : pr) mean += (double)v;
          mean /= (double)bins;
          double shift = (double)dd[c] * tsamp / period * (double)bins;
          for (size_t b = 0; b < bins; ++b) {
            double pos = std::fmod((double)b + shift, (double)bins);
            if (pos < 0.0) pos += (double)bins;
            size_t index = (size_t)std::floor(pos);
            double fraction = pos - (double)index;
            comb[b] += ((double)pr[index % bins] - mean) * (1.0 - fraction) +
                       ((double)pr[(index + 1) % bins] - mean) * fraction;
          }
        }
        double on = -0.0;
        for (size_t i = 0; i < window.width_bins; ++i)
          on += comb[(window.start_bin + i) % bins];
        on /= (double)window.width_bins;
        double tot = -0.0;
        for (double v : comb) tot += v;
        double off = (tot - on * (double)window.width_bins) /
                     (double)(bins - window.width_bins);
        const Cand *match = nullptr;
        for (const Cand &c : members)
          if (std::fabs(c.dm - dm) < step * 0.01 &&
              std::fabs(c.frequency_hz - cand.frequency_hz) < resolution * 1.5)
            if (!match || tcmp64(c.score, match->score) >= 0) match = &c;
        if (ti) r.raw(",");
        r.raw("{");
        r.key("dm"); r.f64(dm); r.raw(",");
        r.key("spectral_score");
        if (match) r.f64(match->score); else r.raw("null");
        r.raw(",");
        r.key("spectral_frequency_hz");
        if (match) r.f64(match->frequency_hz); else r.raw("null");
        r.raw(",");
        r.key("discovery_profile_response"); r.f64(on - off);
        r.raw("}");
      }
      r.raw("]");
      resp = std::move(r.s);
    }
    std::vector<std::string> reasons;
    if (vm.snr < 6.0) reasons.push_back("held-out pulse SNR below threshold");
    size_t np = 0, ns = 0;
    for (auto &m : parts) np += m.snr >= 1.0;
    for (auto &m : subs) ns += m.snr >= 1.0;
    if (np < 3) reasons.push_back("pulse does not persist in enough held-out time segments");
    if (ns < 3) reasons.push_back("pulse does not persist in enough held-out subbands");
    if (best_dm <= 0.0 || contrast < 1.25)
      reasons.push_back("insufficient improvement over zero-DM interference control");
    if (dispersion_widths < 1.5)
      reasons.push_back(
          "dispersion sweep too small relative to selected pulse width to "
          "distinguish local interference");
    if (zero_ratio > 1.0)
      reasons.push_back(
          "stronger rationally related periodic signal in zero-DM discovery control");

    if (fi) j.raw(",");
    j.raw("{");
    j.key("candidate"); json_cand(j, cand); j.raw(",");
    j.key("refined_dm"); j.f64(best_dm); j.raw(",");
    j.key("profile"); json_profile(j, best); j.raw(",");
    j.key("window"); json_window(j, window); j.raw(",");
    j.key("validation"); json_meas(j, vm); j.raw(",");
    j.key("zero_dm_validation"); json_meas(j, zm); j.raw(",");
    j.key("zero_dm_period_s"); j.f64(zero_period); j.raw(",");
    j.key("zero_dm_window"); json_window(j, zw); j.raw(",");
    j.key("dm_contrast"); j.f64(contrast); j.raw(",");
    j.key("dispersion_widths"); j.f64(dispersion_widths); j.raw(",");
    j.key("zero_dm_related_spectral_ratio"); j.f64(zero_ratio); j.raw(",");
    j.key("time_parts"); j.raw("[");
    for (size_t i = 0; i < 4; ++i) { if (i) j.raw(","); json_meas(j, parts[i]); }
    j.raw("],");
    j.key("subbands"); j.raw("[");
    for (size_t i = 0; i < 4; ++i) { if (i) j.raw(","); json_meas(j, subs[i]); }
    j.raw("],");
    j.key("time_profiles"); j.raw("[");
    for (size_t i = 0; i < 4; ++i) {
      if (i) j.raw(",");
      j.raw("[");
      for (size_t b = 0; b < bins; ++b) { if (b) j.raw(","); j.f32(tprof[i].bins[b]); }
      j.raw("]");
    }
    j.raw("],");
    j.key("subband_profiles"); j.raw("[");
    for (size_t i = 0; i < 4; ++i) {
      if (i) j.raw(",");
      j.raw("[");
      for (size_t b = 0; b < bins; ++b) { if (b) j.raw(","); j.f32(sprof[i].bins[b]); }
      j.raw("]");
    }
    j.raw("],");
    j.key("dm_response"); j.raw(resp); j.raw(",");
    j.key("harmonic_members"); j.raw("[");
    for (size_t i = 0; i < members.size(); ++i) { if (i) j.raw(","); json_cand(j, members[i]); }
    j.raw("],");
    j.key("accepted"); j.raw(reasons.empty() ? "true" : "false"); j.raw(",");
    j.key("rejection_reasons"); j.raw("[");
    for (size_t i = 0; i < reasons.size(); ++i) {
      if (i) j.raw(",");
      j.raw("\"" + reasons[i] + "\"");
    }
    j.raw("]}");
  }
  j.raw("]}");
  return true;
}

// ----------------------------------------------------------- fbank
// fbank/src/lib.rs:60-70
bool read_string(const uint8_t *b, size_t len, size_t &pos, std::string &out) {
  if (pos + 4 > len) {
    g_err = "failed to fill whole buffer";
    return false;
  }
  int32_t n;
  std::memcpy(&n, b + pos, 4);
  pos += 4;
  if (n < 1 || n > 4096) {
    g_err = "invalid or unsupported filterbank: bad string length " + std::to_string(n);
    return false;
  }
  if (pos + (size_t)n > len) {
    g_err = "failed to fill whole buffer";
    return false;
  }
  out.assign((const char *)b + pos, (size_t)n);
  pos += (size_t)n;
  return true;
}

struct Field {
  int kind;  // 0 int, 1 float, 2 text
  int32_t i;
  double f;
  std::string t;
};

// fbank/src/lib.rs:72-147
bool parse_header(const uint8_t *b, size_t len, orc_header &h,
                  std::map<std::string, Field> *fields_out = nullptr) {
  size_t pos = 0;
  std::string s;
  if (!read_string(b, len, pos, s)) return false;
  if (s != "HEADER_START") {
    g_err = "invalid or unsupported filterbank: missing HEADER_START";
    return false;
  }
  static const char *ints[] = {"machine_id", "telescope_id", "data_type",
                               "barycentric", "pulsarcentric", "nbits",
                               "nsamples", "nchans", "nifs", "nbeams",
                               "ibeam", "signed"};
  static const char *flts[] = {"az_start", "za_start", "src_raj", "src_dej",
                               "tstart", "tsamp", "fch1", "foff", "refdm",
                               "period"};
  std::map<std::string, Field> fields;
  for (;;) {
    std::string key;
    if (!read_string(b, len, pos, key)) return false;
    if (key == "HEADER_END") break;
    Field f{};
    if (key == "rawdatafile" || key == "source_name") {
      f.kind = 2;
      if (!read_string(b, len, pos, f.t)) return false;
    } else if (std::find_if(std::begin(ints), std::end(ints), [&](const char *k) {
                 return key == k;
               }) != std::end(ints)) {
      if (pos + 4 > len) { g_err = "failed to fill whole buffer"; return false; }
      f.kind = 0;
      std::memcpy(&f.i, b + pos, 4);
      pos += 4;
    } else if (std::find_if(std::begin(flts), std::end(flts), [&](const char *k) {
                 return key == k;
               }) != std::end(flts)) {
      if (pos + 8 > len) { g_err = "failed to fill whole buffer"; return false; }
      f.kind = 1;
      std::memcpy(&f.f, b + pos, 8);
      pos += 8;
    } else {
      g_err = "invalid or unsupported filterbank: unknown keyword " + key +
              "; cannot infer its type safely";
      return false;
    }
    if (fields.count(key)) {
      g_err = "invalid or unsupported filterbank: duplicate " + key;
      return false;
    }
    fields[key] = f;
  }
  auto geti = [&](const char *k, int32_t &v) {
    auto it = fields.find(k);
    if (it == fields.end() || it->second.kind != 0) {
      g_err = std::string("invalid or unsupported filterbank: missing integer ") + k;
      return false;
    }
    v = it->second.i;
    return true;
  };
  auto getf = [&](const char *k, double &v) {
    auto it = fields.find(k);
    if (it == fields.end() || it->second.kind != 1 || !std::isfinite(it->second.f)) {
      g_err = std::string("invalid or unsupported filterbank: missing/invalid float ") + k;
      return false;
    }
    v = it->second.f;
    return true;
  };
  int32_t nchans, nbits;
  double tsamp, fch1, foff;
  if (!geti("nchans", nchans) || !geti("nbits", nbits) || !getf("tsamp", tsamp) ||
      !getf("fch1", fch1) || !getf("foff", foff))
    return false;
  if (nchans <= 0 || tsamp <= 0.0 ||
      !(nbits == 1 || nbits == 2 || nbits == 4 || nbits == 8 || nbits == 16 ||
        nbits == 32)) {
    g_err = "invalid or unsupported filterbank: invalid nchans/tsamp/nbits";
    return false;
  }
  auto it = fields.find("nifs");
  if (it != fields.end() && !(it->second.kind == 0 && it->second.i == 1)) {
    g_err = "invalid or unsupported filterbank: only nifs=1 supported";
    return false;
  }
  it = fields.find("signed");
  if (it != fields.end() && !(it->second.kind == 0 && it->second.i == 0)) {
    g_err = "invalid or unsupported filterbank: signed integer samples unsupported";
    return false;
  }
  it = fields.find("data_type");
  if (it != fields.end() && !(it->second.kind == 0 && it->second.i == 1)) {
    g_err = "invalid or unsupported filterbank: only filterbank data_type=1 supported";
    return false;
  }
  for (int32_t c = 0; c < nchans; ++c) {
    double f = fch1 + (double)c * foff;
    if (!std::isfinite(f) || f <= 0.0) {
      g_err = "invalid or unsupported filterbank: nonpositive frequency";
      return false;
    }
  }
  h.nchans = nchans;
  h.nbits = nbits;
  h.tsamp = tsamp;
  h.fch1 = fch1;
  h.foff = foff;
  h.data_offset = (int64_t)pos;
  if (fields_out) *fields_out = std::move(fields);
  return true;
}

// fbank/src/lib.rs:149-196
bool decode(const uint8_t *b, size_t len, int64_t limit, orc_header &h,
            size_t &nsamples, std::vector<float> *out) {
  if (!parse_header(b, len, h)) return false;
  const uint8_t *payload = b + h.data_offset;
  size_t plen = len - (size_t)h.data_offset;
  size_t bits_per_frame = (size_t)h.nchans * (size_t)h.nbits;
  size_t bits = plen * 8;
  if (bits % bits_per_frame != 0) {
    g_err = "invalid or unsupported filterbank: truncated frame or packed padding unsupported";
    return false;
  }
  size_t total = bits / bits_per_frame;
  size_t ns = limit < 0 ? total : std::min((size_t)limit, total);
  if (ns < 2) {
    g_err = "invalid or unsupported filterbank: need at least two samples";
    return false;
  }
  nsamples = ns;
  if (!out) return true;
  size_t nch = (size_t)h.nchans;
  out->assign(ns * nch, 0.0f);
  for (size_t t = 0; t < ns; ++t)
    for (size_t ch = 0; ch < nch; ++ch) {
      size_t i = t * nch + ch;
      float v;
      switch (h.nbits) {
        case 1: case 2: case 4: {
          size_t bit = i * (size_t)h.nbits;
          v = (float)((payload[bit / 8] >> (bit % 8)) & ((1u << h.nbits) - 1));
          break;
        }
        case 8: v = (float)payload[i]; break;
        case 16: v = (float)(uint16_t)(payload[2 * i] | (payload[2 * i + 1] << 8)); break;
        default: std::memcpy(&v, payload + 4 * i, 4); break;
      }
      if (!std::isfinite(v)) {
        g_err = "invalid or unsupported filterbank: nonfinite sample at " +
                std::to_string(t) + "/" + std::to_string(ch);
        return false;
      }
      (*out)[ch * ns + t] = v;
    }
  return true;
}

Config make_config(const orc_config *c) {
  Config k;
  k.min_hz = c->min_hz;
  k.max_hz = c->max_hz;
  k.threshold = c->threshold;
  k.max_candidates = c->max_candidates;
  k.max_harmonics = c->max_harmonics == 32 ? 32 : 16;
  for (uint64_t i = 0; i < c->nbirdies; ++i)
    k.birdies.push_back({c->birdies[2 * i], c->birdies[2 * i + 1]});
  return k;
}

void to_orc(const Cand &c, orc_candidate &o) {
  o.frequency_hz = c.frequency_hz;
  o.period_s = c.period_s;
  o.dm = c.dm;
  o.harmonics = c.harmonics;
  o.score = c.score;
}

}  // namespace

// ================================================================ C ABI
extern "C" {

const char *orc_last_error(void) { return g_err.c_str(); }

int orc_parse_header(const uint8_t *bytes, uint64_t len, orc_header *out) {
  return parse_header(bytes, len, *out) ? 0 : 1;
}

int orc_decode(const uint8_t *bytes, uint64_t len, int64_t limit,
               orc_header *hdr, uint64_t *nsamples, float *out) {
  orc_header h;
  size_t ns = 0;
  std::vector<float> v;
  if (!decode(bytes, len, limit, h, ns, out ? &v : nullptr)) return 1;
  if (hdr) *hdr = h;
  *nsamples = ns;
  if (out) std::copy(v.begin(), v.end(), out);
  return 0;
}

float orc_median(const float *values, uint64_t n) { return median_f32(values, n); }

// rfi/src/lib.rs:35-43: the channel means and variances of rfi::mask.
int orc_channel_stats(const float *data, uint64_t nchans, uint64_t nsamples, float *means,
                      float *variances) {
  if (nsamples == 0) return fail("channel_stats: empty rows");
  for (uint64_t c = 0; c < nchans; ++c) {
    const float *row = data + c * nsamples;
    const float m = seq_sum_f32(row, nsamples) / (float)nsamples;
    float s = -0.0f;
    for (uint64_t t = 0; t < nsamples; ++t) {
      const float d = row[t] - m;
      s += d * d;
    }
    means[c] = m;
    variances[c] = s / (float)nsamples;
  }
  return 0;
}

int orc_rfi_mask(float *data, uint64_t nchans, uint64_t nsamples,
                 uint64_t block_samples, float threshold, uint64_t *channels,
                 uint64_t *nchannels_bad, uint64_t *blocks, uint64_t blocks_cap,
                 uint64_t *nblocks_bad, double *masked_fraction) {
  if (nsamples == 0 || block_samples == 0 || !std::isfinite(threshold) ||
      threshold <= 0.0f)
    return fail("rfi::mask: invalid arguments");
  Mask m = rfi_mask(data, nsamples, nchans, block_samples, threshold);
  *nchannels_bad = m.channels.size();
  std::copy(m.channels.begin(), m.channels.end(), channels);
  *nblocks_bad = m.blocks.size();
  for (size_t i = 0; i < m.blocks.size() && i < blocks_cap; ++i) blocks[i] = m.blocks[i];
  *masked_fraction = m.masked_fraction;
  return 0;
}

int orc_delays(const double *freqs, uint64_t nchans, double tsamp, double dm,
               uint64_t *out) {
  std::vector<uint64_t> d;
  if (!delays(freqs, nchans, tsamp, dm, d)) return 1;
  std::copy(d.begin(), d.end(), out);
  return 0;
}

int orc_dm_step(const double *freqs, uint64_t nchans, double tsamp, double *out) {
  return dm_step(freqs, nchans, tsamp, *out) ? 0 : 1;
}

int orc_plan(double dm_min, double dm_max, double step, double *out,
             uint64_t cap, uint64_t *n) {
  std::vector<double> t;
  if (!plan(dm_min, dm_max, step, t)) return 1;
  *n = t.size();
  for (size_t i = 0; i < t.size() && i < cap; ++i) out[i] = t[i];
  return 0;
}

int orc_apply(const float *data, uint64_t nchans, uint64_t nsamples,
              const uint64_t *d, int64_t length, float *out, uint64_t *n_out) {
  std::vector<float> x;
  if (!apply(data, nchans, nsamples, d, length, x)) return 1;
  *n_out = x.size();
  if (out) std::copy(x.begin(), x.end(), out);
  return 0;
}

int orc_raw_power(const float *series, uint64_t len, float *out) {
  if (len < 2) return fail("series too short");
  std::vector<float> p = raw_power(series, len);
  std::copy(p.begin(), p.end(), out);
  return 0;
}

int orc_raw_power_f64(const float *series, uint64_t len, double *out) {
  if (len < 2) return fail("series too short");
  std::vector<double> p = raw_power_f64(series, len);
  std::copy(p.begin(), p.end(), out);
  return 0;
}

int orc_periodicity(const float *series, uint64_t len, double tsamp, double dm,
                    const orc_config *cfg, orc_candidate *out, uint64_t cap,
                    uint64_t *n) {
  if (len < 2 || !std::isfinite(tsamp) || tsamp <= 0.0)
    return fail("periodicity: invalid arguments");
  std::vector<Cand> c = periodicity(series, len, tsamp, dm, make_config(cfg));
  *n = c.size();
  for (size_t i = 0; i < c.size() && i < cap; ++i) to_orc(c[i], out[i]);
  return 0;
}

int orc_sift(const orc_candidate *in, uint64_t n, double res, uint64_t limit,
             int reject_dm_zero, orc_candidate *out, uint64_t *n_out) {
  std::vector<Cand> c(n);
  for (size_t i = 0; i < n; ++i)
    c[i] = {in[i].frequency_hz, in[i].period_s, in[i].dm, in[i].harmonics, in[i].score};
  std::vector<Cand> k = sift(c, res, limit, reject_dm_zero != 0);
  *n_out = k.size();
  for (size_t i = 0; i < k.size(); ++i) to_orc(k[i], out[i]);
  return 0;
}

int orc_profile_at(const float *series, uint64_t n, double tsamp, double period,
                   uint64_t bins, uint64_t sample_offset, orc_profile_stats *st,
                   float *values, uint64_t *counts) {
  if (bins < 4 || !std::isfinite(period) || period <= 0.0 || !std::isfinite(tsamp) ||
      tsamp <= 0.0)
    return fail("profile_at: invalid arguments");
  Profile p = profile_at(series, n, tsamp, period, bins, sample_offset);
  st->period_s = p.period_s;
  st->snr = p.snr;
  st->reduced_chi_square = p.rcs;
  std::copy(p.bins.begin(), p.bins.end(), values);
  std::copy(p.counts.begin(), p.counts.end(), counts);
  return 0;
}

int orc_refine(const float *series, uint64_t n, double tsamp, double frequency,
               double span_hz, uint64_t steps, uint64_t bins, orc_profile_stats *st,
               float *values, uint64_t *counts) {
  if (steps == 0 || !(frequency > span_hz) || !(span_hz >= 0.0))
    return fail("refine: invalid arguments");
  Profile p = refine(series, n, tsamp, frequency, span_hz, steps, bins);
  st->period_s = p.period_s;
  st->snr = p.snr;
  st->reduced_chi_square = p.rcs;
  std::copy(p.bins.begin(), p.bins.end(), values);
  std::copy(p.counts.begin(), p.counts.end(), counts);
  return 0;
}

int orc_measure(const float *x, uint64_t n, uint64_t offset, double tsamp,
                double period, uint64_t start_bin, uint64_t width_bins,
                uint64_t bins, orc_measurement *out) {
  Window w{start_bin, width_bins, bins};
  Measurement m = measure(x, n, offset, tsamp, period, w);
  out->snr = m.snr;
  out->on_samples = m.on;
  out->off_samples = m.off;
  out->mean_difference = m.diff;
  out->standard_error = m.err;
  return 0;
}

int orc_search_trials(const float *data, uint64_t nchans, uint64_t nsamples,
                      const double *freqs, double tsamp, const double *trials,
                      uint64_t ntrials, uint64_t discovery, const orc_config *cfg,
                      int threads, uint64_t *counts, orc_candidate *out,
                      uint64_t cap, uint64_t *n_total) {
  std::string err;
  auto lists = search_trials(data, nchans, nsamples, freqs, tsamp, trials, ntrials,
                             discovery, make_config(cfg), threads, err);
  if (!err.empty()) return fail(err);
  uint64_t k = 0;
  for (size_t i = 0; i < ntrials; ++i) {
    if (counts) counts[i] = lists[i].size();
    for (const Cand &c : lists[i]) {
      if (k < cap) to_orc(c, out[k]);
      ++k;
    }
  }
  *n_total = k;
  return 0;
}

char *orc_psr_search_json(const uint8_t *bytes, uint64_t len, double dm_min,
                          double dm_max, double dm_step_arg, double min_hz,
                          double max_hz, double threshold, uint64_t top,
                          uint64_t bins, int no_rfi, const double *birdies,
                          uint64_t nbirdies, int64_t max_samples, int threads) {
  // cli/src/main.rs:380-571 without plots, hashing and file output.
  if (!std::isfinite(min_hz) || !std::isfinite(max_hz) || min_hz <= 0.0 ||
      max_hz <= min_hz || !std::isfinite(threshold) || threshold <= 0.0 || top == 0 ||
      bins < 8) {
    g_err = "invalid search settings";
    return nullptr;
  }
  orc_header h;
  size_t ns = 0;
  std::vector<float> data;
  if (!decode(bytes, len, max_samples, h, ns, &data)) return nullptr;
  size_t nch = (size_t)h.nchans;
  std::vector<double> freqs(nch);
  for (size_t c = 0; c < nch; ++c) freqs[c] = h.fch1 + (double)c * h.foff;
  double tsamp = h.tsamp;
  Mask mask;
  if (!no_rfi) {
    size_t block = std::max<size_t>((size_t)(0.1 / tsamp), 32);
    mask = rfi_mask(data.data(), ns, nch, block, 8.0f);
  }
  double step = dm_step_arg;
  if (!(step > 0.0) && !dm_step(freqs.data(), nch, tsamp, step)) return nullptr;
  std::vector<double> trials;
  if (!plan(dm_min, dm_max, step, trials)) return nullptr;
  std::vector<uint64_t> dmx;
  if (!delays(freqs.data(), nch, tsamp, dm_max, dmx)) return nullptr;
  uint64_t max_delay = *std::max_element(dmx.begin(), dmx.end());
  if (max_delay > ns || ns - max_delay < 512) {
    g_err = "DM range leaves fewer than 512 samples";
    return nullptr;
  }
  size_t length = ns - max_delay;
  if (max_delay > length || length - max_delay < 256) {
    g_err = "DM range leaves no independent discovery/confirmation split";
    return nullptr;
  }
  size_t discovery = (length - max_delay) / 2;
  Config cfg;
  cfg.min_hz = min_hz;
  cfg.max_hz = max_hz;
  cfg.threshold = threshold;
  cfg.max_candidates = 32;
  for (uint64_t i = 0; i < nbirdies; ++i)
    cfg.birdies.push_back({birdies[2 * i], birdies[2 * i + 1]});
  std::string err;
  auto lists = search_trials(data.data(), nch, ns, freqs.data(), tsamp, trials.data(),
                             trials.size(), discovery, cfg, threads, err);
  if (!err.empty()) {
    g_err = err;
    return nullptr;
  }
  std::vector<Cand> all;
  for (auto &l : lists) all.insert(all.end(), l.begin(), l.end());
  Json conf;
  if (!analyze(data.data(), ns, freqs, tsamp, trials, all, top, bins, conf)) return nullptr;

  Json j;
  j.raw("{");
  j.key("schema_version"); j.raw("2,");
  j.key("confirmation"); j.raw(conf.s); j.raw(",");
  j.key("sample_count"); j.u64(ns); j.raw(",");
  j.key("tsamp"); j.f64(tsamp); j.raw(",");
  j.key("dm_min"); j.f64(dm_min); j.raw(",");
  j.key("dm_max"); j.f64(dm_max); j.raw(",");
  j.key("dm_step"); j.f64(step); j.raw(",");
  j.key("trial_count"); j.u64(trials.size()); j.raw(",");
  j.key("common_samples"); j.u64(length); j.raw(",");
  j.key("discovery_samples_search"); j.u64(discovery); j.raw(",");
  j.key("threads"); j.u64((uint64_t)std::max(threads, 1)); j.raw(",");
  j.key("min_hz"); j.f64(min_hz); j.raw(",");
  j.key("max_hz"); j.f64(max_hz); j.raw(",");
  j.key("threshold"); j.f64(threshold); j.raw(",");
  j.key("birdies"); j.raw("[");
  for (uint64_t i = 0; i < nbirdies; ++i) {
    if (i) j.raw(",");
    j.raw("[");
    j.f64(birdies[2 * i]);
    j.raw(",");
    j.f64(birdies[2 * i + 1]);
    j.raw("]");
  }
  j.raw("],");
  j.key("rfi");
  if (no_rfi) {
    j.raw("null");
  } else {
    j.raw("{");
    j.key("channels"); j.raw("[");
    for (size_t i = 0; i < mask.channels.size(); ++i) { if (i) j.raw(","); j.u64(mask.channels[i]); }
    j.raw("],");
    j.key("blocks"); j.raw("[");
    for (size_t i = 0; i < mask.blocks.size(); ++i) { if (i) j.raw(","); j.u64(mask.blocks[i]); }
    j.raw("],");
    j.key("block_samples"); j.u64(mask.block_samples); j.raw(",");
    j.key("masked_fraction"); j.f64(mask.masked_fraction);
    j.raw("}");
  }
  j.raw(",");
  j.key("trial_candidate_counts"); j.raw("[");
  for (size_t i = 0; i < lists.size(); ++i) { if (i) j.raw(","); j.u64(lists[i].size()); }
  j.raw("],");
  j.key("all_candidates"); j.raw("[");
  for (size_t i = 0; i < all.size(); ++i) { if (i) j.raw(","); json_cand(j, all[i]); }
  j.raw("]}");
  char *res = (char *)std::malloc(j.s.size() + 1);
  std::memcpy(res, j.s.c_str(), j.s.size() + 1);
  return res;
}

// confirmation::analyze (confirmation.rs:203-496) alone, on already masked
// channel-major data and a given candidate list; the Outcome JSON.
char *orc_analyze_json(const float *data, uint64_t nchans, uint64_t nsamples,
                       const double *freqs, double tsamp, const double *trials,
                       uint64_t ntrials, const orc_candidate *generated, uint64_t ngenerated,
                       uint64_t limit, uint64_t bins) {
  std::vector<double> f(freqs, freqs + nchans), t(trials, trials + ntrials);
  std::vector<Cand> gen(ngenerated);
  for (uint64_t i = 0; i < ngenerated; ++i)
    gen[i] = Cand{generated[i].frequency_hz, generated[i].period_s, generated[i].dm,
                  generated[i].harmonics, generated[i].score};
  Json j;
  if (!analyze(data, nsamples, f, tsamp, t, gen, limit, bins, j)) return nullptr;
  char *res = (char *)std::malloc(j.s.size() + 1);
  std::memcpy(res, j.s.c_str(), j.s.size() + 1);
  return res;
}

// FP64 reference of the gradient-refinement objective and its gradient (a
// model this project defines; the reference has no counterpart).  Every
// quantity is f64: fractional delays a_c, the interpolated series y and
// z = dy/dDM, cloud-in-cell folding, J = sum_b (p_b - mean)^2 / (n v), and the
// analytic derivatives d/dP, d/dPdot, d/dDM of J with v held fixed.
int orc_refine_objective(const float *data, uint64_t nch, uint64_t ns, const double *freqs,
                         double tsamp, uint64_t n, double P, double Pdot, double DM,
                         uint64_t bins, uint64_t subints, double variance, double *J,
                         double *grad, double *profile) {
  if (n + 2 > ns || bins < 4 || subints < 1 || !(P > 0.0) || !(DM >= 0.0)) {
    g_err = "refine_objective: invalid arguments";
    return 1;
  }
  double fmax = 0.0;
  for (uint64_t c = 0; c < nch; ++c) fmax = std::fmax(fmax, freqs[c]);
  std::vector<double> a(nch), k(nch);
  std::vector<uint64_t> m(nch);
  for (uint64_t c = 0; c < nch; ++c) {
    k[c] = 4148.808 * (1.0 / (freqs[c] * freqs[c]) - 1.0 / (fmax * fmax)) / tsamp;
    const double tau = k[c] * DM;
    m[c] = (uint64_t)std::floor(tau);
    a[c] = tau - std::floor(tau);
    if (m[c] + n + 1 > ns) {
      g_err = "refine_objective: delays leave fewer than n + 1 samples";
      return 1;
    }
  }
  std::vector<double> y(n, 0.0), z(n, 0.0);
  for (uint64_t c = 0; c < nch; ++c) {
    const float *row = data + c * ns + m[c];
    for (uint64_t t = 0; t < n; ++t) {
      const double v0 = row[t], v1 = row[t + 1];
      y[t] += (1.0 - a[c]) * v0 + a[c] * v1;
      z[t] += k[c] * (v1 - v0);
    }
  }
  double mean = 0.0, sq = 0.0;
  for (double v : y) {
    mean += v;
    sq += v * v;
  }
  mean /= (double)n;
  const double v = variance > 0.0 ? variance : std::fmax(sq / (double)n - mean * mean, 1e-300);
  const double nu = 1.0 / P, nudot = -Pdot / (P * P);
  const double B = (double)bins;
  std::vector<double> p(bins, 0.0);
  std::vector<uint64_t> b0s(n), b1s(n);
  std::vector<double> ws(n);
  for (uint64_t t = 0; t < n; ++t) {
    const double T = (double)t * tsamp;
    const double ph = nu * T + 0.5 * nudot * T * T;
    const double u = (ph - std::floor(ph)) * B;
    double fb = std::floor(u);
    uint64_t b0 = (uint64_t)fb;
    double w = u - fb;
    if (b0 >= bins) {
      b0 = 0;
      w = 0.0;
    }
    const uint64_t b1 = b0 + 1 == bins ? 0 : b0 + 1;
    b0s[t] = b0;
    b1s[t] = b1;
    ws[t] = w;
    p[b0] += (1.0 - w) * y[t];
    p[b1] += w * y[t];
  }
  double pm = 0.0;
  for (double x : p) pm += x;
  pm /= B;
  double j = 0.0;
  std::vector<double> g(bins);
  for (uint64_t b = 0; b < bins; ++b) {
    const double d = p[b] - pm;
    j += d * d;
    g[b] = 2.0 * d / ((double)n * v);
  }
  *J = j / ((double)n * v);
  double dnu = 0.0, dnudot = 0.0, ddm = 0.0;
  for (uint64_t t = 0; t < n; ++t) {
    const double T = (double)t * tsamp;
    const double du = y[t] * (g[b1s[t]] - g[b0s[t]]);
    dnu += du * B * T;
    dnudot += du * B * 0.5 * T * T;
    ddm += ((1.0 - ws[t]) * g[b0s[t]] + ws[t] * g[b1s[t]]) * z[t];
  }
  if (grad) {
    grad[0] = dnu * (-1.0 / (P * P)) + dnudot * (2.0 * Pdot / (P * P * P));
    grad[1] = dnudot * (-1.0 / (P * P));
    grad[2] = ddm;
  }
  if (profile) std::copy(p.begin(), p.end(), profile);
  return 0;
}

void orc_free(void *p) { std::free(p); }

}  // extern "C"
