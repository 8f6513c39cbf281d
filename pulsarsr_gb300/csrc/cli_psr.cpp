// psr — the reference's command line (crates/cli/src/main.rs) on libpsr.
//
//   psr header FILE
//   psr fold FILE --period P --dm DM [--bins 64] [--out output_fold]
//   psr dedisperse FILE --dm DM [--out output]
//   psr inspect FILE [--out output] [--max-samples N]
//   psr synth FILE [--samples 65536] [--channels 32] [--tsamp 0.00025]
//              [--period 0.032] [--dm 62] [--amplitude 0.5] [--duty 0.05] [--seed 42]
//   psr search FILE [--dm-min 0] [--dm-max 500] [--dm-step S] [--min-hz 15]
//              [--max-hz 2000] [--threshold 8] [--top 5] [--bins 64] [--no-rfi]
//              [--birdie HZ:HALF_WIDTH_HZ]... [--max-samples N] [--threads N]
//              [--out output]
//
// The JSON files have the reference's names, fields, field order and number
// format (header.json, report.json schema 2, series.json, fold.json).  PNG
// plots are not written: this build has no plotting backend.
#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "json_writer.h"
#include "psr.h"

using psrjson::Value;

namespace {

struct Fail : std::runtime_error {
  using std::runtime_error::runtime_error;
};

std::string last_error() {
  char buf[4096];
  psr_last_error(buf, sizeof buf);
  return buf;
}

void check(int rc) {
  if (rc != PSR_OK) throw Fail(last_error());
}

std::vector<uint8_t> read_file(const std::string &path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw Fail("No such file or directory (os error 2)");
  std::vector<uint8_t> b((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  return b;
}

void make_dirs(const std::string &path) {
  std::string cur;
  std::stringstream ss(path);
  std::string part;
  if (!path.empty() && path[0] == '/') cur = "/";
  while (std::getline(ss, part, '/')) {
    if (part.empty()) continue;
    cur += part + "/";
    mkdir(cur.c_str(), 0755);
  }
  struct stat st;
  if (stat(path.c_str(), &st) != 0 || !S_ISDIR(st.st_mode))
    throw Fail("cannot create output directory " + path);
}

std::string join(const std::string &dir, const std::string &name) {
  return dir.empty() || dir.back() == '/' ? dir + name : dir + "/" + name;
}

void write_json(const std::string &path, const Value &v) {
  std::ofstream f(path, std::ios::binary);
  if (!f) throw Fail("cannot write " + path);
  f << psrjson::dump(v, true);
}

// ---------------------------------------------------------------- SHA-256
// FIPS 180-4.  The round constants are the first 32 fractional bits of the
// cube roots of the first 64 primes and the initial hash the first 32
// fractional bits of the square roots of the first 8 primes; both are
// computed here with exact integer roots.
struct Sha256 {
  uint32_t k[64], h[8];
  uint64_t total = 0;
  uint8_t block[64];
  size_t used = 0;

  static unsigned __int128 iroot(unsigned __int128 v, int n) {
    // Roots here are below 2^36, so mid^n stays below 2^108.
    unsigned __int128 lo = 0, hi = (unsigned __int128)1 << 36;
    while (lo < hi) {
      const unsigned __int128 mid = (lo + hi + 1) / 2;
      unsigned __int128 p = mid;
      for (int i = 1; i < n; ++i) p *= mid;
      if (p <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
  }
  Sha256() {
    int primes[64], np = 0;
    for (int c = 2; np < 64; ++c) {
      bool prime = true;
      for (int d = 2; d * d <= c; ++d) prime = prime && (c % d != 0);
      if (prime) primes[np++] = c;
    }
    for (int i = 0; i < 64; ++i)
      k[i] = (uint32_t)iroot((unsigned __int128)primes[i] << 96, 3);
    for (int i = 0; i < 8; ++i) h[i] = (uint32_t)iroot((unsigned __int128)primes[i] << 64, 2);
  }
  static uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }
  void compress(const uint8_t *p) {
    uint32_t w[64];
    for (int i = 0; i < 16; ++i)
      w[i] = (uint32_t)p[4 * i] << 24 | (uint32_t)p[4 * i + 1] << 16 |
             (uint32_t)p[4 * i + 2] << 8 | (uint32_t)p[4 * i + 3];
    for (int i = 16; i < 64; ++i) {
      const uint32_t s0 = rotr(w[i - 15], 7) ^ rotr(w[i - 15], 18) ^ (w[i - 15] >> 3);
      const uint32_t s1 = rotr(w[i - 2], 17) ^ rotr(w[i - 2], 19) ^ (w[i - 2] >> 10);
      w[i] = w[i - 16] + s0 + w[i - 7] + s1;
    }
    uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4], f = h[5], g = h[6], hh = h[7];
    for (int i = 0; i < 64; ++i) {
      const uint32_t S1 = rotr(e, 6) ^ rotr(e, 11) ^ rotr(e, 25);
      const uint32_t ch = (e & f) ^ (~e & g);
      const uint32_t t1 = hh + S1 + ch + k[i] + w[i];
      const uint32_t S0 = rotr(a, 2) ^ rotr(a, 13) ^ rotr(a, 22);
      const uint32_t mj = (a & b) ^ (a & c) ^ (b & c);
      const uint32_t t2 = S0 + mj;
      hh = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
    }
    h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e; h[5] += f; h[6] += g; h[7] += hh;
  }
  void update(const uint8_t *p, size_t n) {
    total += n;
    while (n) {
      const size_t t = std::min(n, 64 - used);
      std::memcpy(block + used, p, t);
      used += t; p += t; n -= t;
      if (used == 64) {
        compress(block);
        used = 0;
      }
    }
  }
  std::string hex() {
    const uint64_t bits = total * 8;
    const uint8_t one = 0x80, zero = 0;
    update(&one, 1);
    while (used != 56) update(&zero, 1);
    uint8_t len[8];
    for (int i = 0; i < 8; ++i) len[i] = (uint8_t)(bits >> (56 - 8 * i));
    update(len, 8);
    char out[65];
    for (int i = 0; i < 8; ++i) std::snprintf(out + 8 * i, 9, "%08x", h[i]);
    return std::string(out, 64);
  }
};

// ------------------------------------------------------------- arguments
struct Args {
  std::string cmd, file;
  std::map<std::string, std::string> opt;
  std::vector<std::string> birdies;
  bool no_rfi = false;
  bool has(const std::string &k) const { return opt.count(k) > 0; }
  double num(const std::string &k, double dflt) const {
    auto it = opt.find(k);
    if (it == opt.end()) return dflt;
    char *end = nullptr;
    const double v = std::strtod(it->second.c_str(), &end);
    if (!end || *end) throw Fail("invalid value '" + it->second + "' for '--" + k + "'");
    return v;
  }
  uint64_t count(const std::string &k, uint64_t dflt) const {
    auto it = opt.find(k);
    if (it == opt.end()) return dflt;
    char *end = nullptr;
    const unsigned long long v = std::strtoull(it->second.c_str(), &end, 10);
    if (!end || *end || it->second[0] == '-')
      throw Fail("invalid value '" + it->second + "' for '--" + k + "'");
    return v;
  }
};

Args parse_args(int argc, char **argv) {
  Args a;
  if (argc < 2)
    throw Fail("usage: psr <header|fold|dedisperse|inspect|search|synth> FILE [options]");
  a.cmd = argv[1];
  for (int i = 2; i < argc; ++i) {
    std::string s = argv[i];
    if (s.rfind("--", 0) == 0) {
      std::string k = s.substr(2), v;
      const size_t eq = k.find('=');
      if (eq != std::string::npos) {
        v = k.substr(eq + 1);
        k = k.substr(0, eq);
      } else if (k != "no-rfi") {
        if (i + 1 >= argc) throw Fail("a value is required for '--" + k + "'");
        v = argv[++i];
      }
      for (char &c : k)
        if (c == '_') c = '-';
      if (k == "no-rfi") a.no_rfi = true;
      else if (k == "birdie") a.birdies.push_back(v);
      else a.opt[k] = v;
    } else if (a.file.empty()) {
      a.file = s;
    } else {
      throw Fail("unexpected argument '" + s + "'");
    }
  }
  if (a.file.empty()) throw Fail("the FILE argument is required");
  return a;
}

// ------------------------------------------------------------ filterbank
struct Fb {
  psr_fb *fb = nullptr;
  psr_header h{};
  uint64_t ns = 0;
  std::vector<uint8_t> bytes;
  ~Fb() {
    if (fb) psr_fb_free(fb);
  }
  std::vector<double> freqs() const {
    std::vector<double> f((size_t)h.nchans);
    for (int64_t c = 0; c < h.nchans; ++c) f[(size_t)c] = h.fch1 + (double)c * h.foff;
    return f;
  }
};

void open_fb(Fb &fb, const std::string &path, int64_t limit) {
  check(psr_fb_read(path.c_str(), limit, &fb.fb));
  check(psr_fb_info(fb.fb, &fb.h, &fb.ns));
  // The header bytes (for header.json): SIGPROC headers are short.
  std::ifstream f(path, std::ios::binary);
  fb.bytes.resize((size_t)fb.h.data_offset);
  f.read(reinterpret_cast<char *>(fb.bytes.data()), (std::streamsize)fb.bytes.size());
}

Value header_value(const std::vector<uint8_t> &bytes) {
  uint64_t need = 0;
  check(psr_header_json(bytes.data(), bytes.size(), 0, nullptr, 0, &need));
  std::string s(need + 1, '\0');
  check(psr_header_json(bytes.data(), bytes.size(), 0, &s[0], s.size(), &need));
  s.resize(need);
  Value v;
  if (!psrjson::parse(s, v)) throw Fail("internal: header JSON");
  return v;
}

std::vector<uint64_t> delays_for(const Fb &fb, double dm) {
  std::vector<double> f = fb.freqs();
  std::vector<uint64_t> d(f.size());
  check(psr_delays(f.data(), f.size(), fb.h.tsamp, dm, d.data()));
  return d;
}

std::vector<float> dedisperse(const Fb &fb, const std::vector<uint64_t> &d, int64_t length) {
  uint64_t n = 0;
  check(psr_dedisperse(fb.fb, d.data(), length, nullptr, 0, &n));
  std::vector<float> x(n);
  check(psr_dedisperse(fb.fb, d.data(), length, x.data(), x.size(), &n));
  return x;
}

// Numbers inside serde_json::json!{} become f64 (f32 profile bins included)
// and object keys are sorted.
Value profile_value_sorted(const psr_profile_stats &st, const std::vector<float> &v,
                           const std::vector<uint64_t> &c) {
  Value p = Value::object();
  Value b = Value::array(), n = Value::array();
  for (float x : v) b.push(Value::num((double)x));
  for (uint64_t x : c) n.push(Value::u64(x));
  p.set("bins", std::move(b));
  p.set("counts", std::move(n));
  p.set("period_s", Value::num(st.period_s));
  p.set("reduced_chi_square", Value::num(st.reduced_chi_square));
  p.set("snr", Value::num(st.snr));
  return p;
}

// -------------------------------------------------------------- commands
int cmd_header(const Args &a) {
  std::printf("%s\n", psrjson::dump(header_value(read_file(a.file)), true).c_str());
  return 0;
}

// main.rs:295-331
int cmd_fold(const Args &a) {
  if (!a.has("period")) throw Fail("the argument '--period <PERIOD>' is required");
  if (!a.has("dm")) throw Fail("the argument '--dm <DM>' is required");
  const double period = a.num("period", 0), dm = a.num("dm", 0);
  const uint64_t bins = a.count("bins", 64);
  const std::string out = a.has("out") ? a.opt.at("out") : "output_fold";
  if (!std::isfinite(period) || period <= 0.0 || bins < 8)
    throw Fail("positive period and >=8 bins required");
  Fb fb;
  open_fb(fb, a.file, -1);
  const std::vector<float> x = dedisperse(fb, delays_for(fb, dm), -1);
  psr_profile_stats st{};
  std::vector<float> vals(bins);
  std::vector<uint64_t> cnts(bins);
  check(psr_profile_at(x.data(), x.size(), fb.h.tsamp, period, bins, 0, &st, vals.data(),
                       cnts.data()));
  make_dirs(out);
  Value j = Value::object();
  j.set("dm", Value::num(dm));
  j.set("input", Value::str(a.file));
  j.set("profile", profile_value_sorted(st, vals, cnts));
  j.set("searched", Value::boolean(false));
  write_json(join(out, "fold.json"), j);
  return 0;
}

// main.rs:368-379
int cmd_dedisperse(const Args &a) {
  if (!a.has("dm")) throw Fail("the argument '--dm <DM>' is required");
  const double dm = a.num("dm", 0);
  const std::string out = a.has("out") ? a.opt.at("out") : "output";
  make_dirs(out);
  Fb fb;
  open_fb(fb, a.file, -1);
  const std::vector<uint64_t> d = delays_for(fb, dm);
  const std::vector<float> x = dedisperse(fb, d, -1);
  {
    std::ofstream f(join(out, "series.f32"), std::ios::binary);
    for (float v : x) {
      uint8_t b[4];
      uint32_t u;
      std::memcpy(&u, &v, 4);
      for (int i = 0; i < 4; ++i) b[i] = (uint8_t)(u >> (8 * i));
      f.write(reinterpret_cast<const char *>(b), 4);
    }
  }
  Value dl = Value::array();
  for (uint64_t v : d) dl.push(Value::u64(v));
  Value j = Value::object();
  j.set("delays", std::move(dl));
  j.set("dm", Value::num(dm));
  j.set("dtype", Value::str("little-endian float32"));
  j.set("normalization", Value::str("raw channel sum"));
  j.set("samples", Value::u64(x.size()));
  j.set("tsamp", Value::num(fb.h.tsamp));
  write_json(join(out, "series.json"), j);
  return 0;
}

// main.rs:191-196 (header.json; the waterfall and DM-0 PNGs are not drawn)
int cmd_inspect(const Args &a) {
  const std::string out = a.has("out") ? a.opt.at("out") : "output";
  Fb fb;
  open_fb(fb, a.file, a.has("max-samples") ? (int64_t)a.count("max-samples", 0) : -1);
  make_dirs(out);
  write_json(join(out, "header.json"), header_value(fb.bytes));
  return 0;
}

// main.rs:341-367 and fbank::write (fbank/src/lib.rs:216-250): a 32-bit
// filterbank (keywords in sorted order, time-major samples) and
// FILE.truth.json with the configuration.  The samples come from the device
// generator (psr_fb_synth): same signal model and header, different noise
// stream than the reference's ChaCha8 generator.
int cmd_synth(const Args &a) {
  const uint64_t samples = a.count("samples", 65536), channels = a.count("channels", 32);
  const double tsamp = a.num("tsamp", 0.00025), period = a.num("period", 0.032);
  const double dm = a.num("dm", 62.0), amplitude = a.num("amplitude", 0.5);
  const double duty = a.num("duty", 0.05);
  const uint64_t seed = a.count("seed", 42);
  const double fch1 = 1450.0, foff = -4.0;
  if (samples < 2 || channels < 1 || !std::isfinite(period) || period <= 0.0 ||
      !std::isfinite(duty) || duty <= 0.0 || duty >= 0.5 || !std::isfinite(amplitude) ||
      amplitude < 0.0)
    throw Fail("invalid synthetic configuration");
  {
    std::vector<double> f(channels);
    for (uint64_t c = 0; c < channels; ++c) f[c] = fch1 + (double)c * foff;
    std::vector<uint64_t> d(channels);
    check(psr_delays(f.data(), f.size(), tsamp, dm, d.data()));
  }
  psr_synth_pulsar p{period, 0.0, dm, duty, amplitude, 0.25};
  psr_synth_config cfg{(int64_t)channels, 32, samples, tsamp, fch1, foff, seed,
                       100.0, 1.0, 0.0, &p, 1};
  psr_fb *fb = nullptr;
  check(psr_fb_synth(&cfg, &fb));
  std::vector<float> data(channels * samples);
  const int rc = psr_fb_download(fb, data.data());
  psr_fb_free(fb);
  check(rc);
  std::ofstream f(a.file, std::ios::binary);
  if (!f) throw Fail("cannot write " + a.file);
  auto put_i32 = [&](int32_t v) {
    uint8_t b[4];
    for (int i = 0; i < 4; ++i) b[i] = (uint8_t)((uint32_t)v >> (8 * i));
    f.write(reinterpret_cast<const char *>(b), 4);
  };
  auto put_f64 = [&](double v) {
    uint64_t u;
    std::memcpy(&u, &v, 8);
    uint8_t b[8];
    for (int i = 0; i < 8; ++i) b[i] = (uint8_t)(u >> (8 * i));
    f.write(reinterpret_cast<const char *>(b), 8);
  };
  auto put_str = [&](const std::string &t) {
    put_i32((int32_t)t.size());
    f.write(t.data(), (std::streamsize)t.size());
  };
  put_str("HEADER_START");
  // BTreeMap order: data_type, fch1, foff, nbits, nchans, nifs, signed,
  // source_name, tsamp.
  put_str("data_type"); put_i32(1);
  put_str("fch1"); put_f64(fch1);
  put_str("foff"); put_f64(foff);
  put_str("nbits"); put_i32(32);
  put_str("nchans"); put_i32((int32_t)channels);
  put_str("nifs"); put_i32(1);
  put_str("signed"); put_i32(0);
  put_str("source_name"); put_str("seeded synthetic pulsar");
  put_str("tsamp"); put_f64(tsamp);
  put_str("HEADER_END");
  std::vector<uint8_t> frame(channels * 4);
  for (uint64_t t = 0; t < samples; ++t) {
    for (uint64_t c = 0; c < channels; ++c) {
      uint32_t u;
      std::memcpy(&u, &data[c * samples + t], 4);
      for (int i = 0; i < 4; ++i) frame[c * 4 + i] = (uint8_t)(u >> (8 * i));
    }
    f.write(reinterpret_cast<const char *>(frame.data()), (std::streamsize)frame.size());
  }
  f.close();
  std::string truth = a.file;
  const size_t dot = truth.find_last_of('.'), slash = truth.find_last_of('/');
  if (dot != std::string::npos && (slash == std::string::npos || dot > slash))
    truth = truth.substr(0, dot);
  truth += ".truth.json";
  Value j = Value::object();
  j.set("nsamples", Value::u64(samples));
  j.set("nchans", Value::u64(channels));
  j.set("tsamp", Value::num(tsamp));
  j.set("fch1", Value::num(fch1));
  j.set("foff", Value::num(foff));
  j.set("period_s", Value::num(period));
  j.set("dm", Value::num(dm));
  j.set("duty_cycle", Value::num(duty));
  j.set("amplitude", Value::num(amplitude));
  j.set("seed", Value::u64(seed));
  write_json(truth, j);
  std::printf("Wrote %s and truth metadata\n", a.file.c_str());
  return 0;
}

std::string fixed(double v, int prec) {
  char b[64];
  std::snprintf(b, sizeof b, "%.*f", prec, v);
  return b;
}

// main.rs:380-571
int cmd_search(const Args &a) {
  const auto start = std::chrono::steady_clock::now();
  const double dm_min = a.num("dm-min", 0.0), dm_max = a.num("dm-max", 500.0);
  const double min_hz = a.num("min-hz", 15.0), max_hz = a.num("max-hz", 2000.0);
  const double threshold = a.num("threshold", 8.0);
  const uint64_t top = a.count("top", 5), bins = a.count("bins", 64);
  const std::string out = a.has("out") ? a.opt.at("out") : "output";
  std::vector<double> birdies;
  for (const std::string &b : a.birdies) {
    const size_t c = b.find(':');
    if (c == std::string::npos) throw Fail("invalid value '" + b + "' for '--birdie': expected HZ:HALF_WIDTH_HZ");
    char *e1 = nullptr, *e2 = nullptr;
    const std::string hz = b.substr(0, c), hw = b.substr(c + 1);
    const double f = std::strtod(hz.c_str(), &e1), w = std::strtod(hw.c_str(), &e2);
    if (*e1 || hz.empty()) throw Fail("invalid value '" + b + "' for '--birdie': invalid frequency");
    if (*e2 || hw.empty()) throw Fail("invalid value '" + b + "' for '--birdie': invalid width");
    if (!std::isfinite(f) || !std::isfinite(w) || f < 0 || w < 0)
      throw Fail("invalid value '" + b + "' for '--birdie': nonnegative finite birdie required");
    birdies.push_back(f);
    birdies.push_back(w);
  }
  if (!std::isfinite(min_hz) || !std::isfinite(max_hz) || min_hz <= 0.0 || max_hz <= min_hz ||
      !std::isfinite(threshold) || threshold <= 0.0 || top == 0 || bins < 8)
    throw Fail("invalid search settings");
  uint64_t threads = std::thread::hardware_concurrency();
  if (a.has("threads")) {
    threads = a.count("threads", 0);
    if (threads == 0) throw Fail("threads must be positive");
  }
  make_dirs(out);
  Fb fb;
  open_fb(fb, a.file, a.has("max-samples") ? (int64_t)a.count("max-samples", 0) : -1);
  const std::vector<double> freqs = fb.freqs();
  const double tsamp = fb.h.tsamp;
  write_json(join(out, "header.json"), header_value(fb.bytes));
  Value rfi = Value::null();
  if (!a.no_rfi) {
    const uint64_t block = std::max<uint64_t>((uint64_t)(0.1 / tsamp), 32);
    std::vector<uint64_t> ch((size_t)fb.h.nchans), bl(fb.ns / block + 2);
    uint64_t nc = 0, nb = 0;
    double frac = 0.0;
    check(psr_rfi_mask(fb.fb, block, 8.0f, ch.data(), &nc, bl.data(), bl.size(), &nb, &frac));
    Value c = Value::array(), b = Value::array();
    for (uint64_t i = 0; i < nc; ++i) c.push(Value::u64(ch[i]));
    for (uint64_t i = 0; i < nb; ++i) b.push(Value::u64(bl[i]));
    rfi = Value::object();
    rfi.set("channels", std::move(c));
    rfi.set("blocks", std::move(b));
    rfi.set("block_samples", Value::u64(block));
    rfi.set("masked_fraction", Value::num(frac));
  }
  double step = 0.0;
  if (a.has("dm-step")) step = a.num("dm-step", 0.0);
  else check(psr_dm_step(freqs.data(), freqs.size(), tsamp, &step));
  uint64_t nt = 0;
  int rc = psr_plan(dm_min, dm_max, step, nullptr, 0, &nt);
  if (rc != PSR_OK && rc != PSR_ECAPACITY) check(rc);
  std::vector<double> trials(nt);
  check(psr_plan(dm_min, dm_max, step, trials.data(), trials.size(), &nt));
  const std::vector<uint64_t> dmax = delays_for(fb, dm_max);
  uint64_t max_delay = 0;
  for (uint64_t d : dmax) max_delay = std::max(max_delay, d);
  if (max_delay > fb.ns || fb.ns - max_delay < 512)
    throw Fail("DM range leaves fewer than 512 samples");
  const uint64_t length = fb.ns - max_delay;
  if (max_delay > length || length - max_delay < 256)
    throw Fail("DM range leaves no independent discovery/confirmation split");
  const uint64_t discovery = (length - max_delay) / 2;
  psr_search_config cfg{min_hz, max_hz, threshold, 32,
                        birdies.empty() ? nullptr : birdies.data(), birdies.size() / 2, 16};
  std::printf("%llu samples, %lld channels, %llu DM trials (step %s), %llu threads\n",
              (unsigned long long)fb.ns, (long long)fb.h.nchans, (unsigned long long)nt,
              fixed(step, 6).c_str(), (unsigned long long)threads);
  std::vector<uint64_t> counts(nt);
  uint64_t total = 0;
  std::vector<psr_candidate> all(nt * cfg.max_candidates);
  check(psr_search_trials(fb.fb, trials.data(), nt, discovery, &cfg, counts.data(), all.data(),
                          all.size(), &total));
  all.resize(total);
  psr_outcome *oc = nullptr;
  check(psr_analyze(fb.fb, trials.data(), nt, all.data(), all.size(), top, bins, nullptr, &oc));
  std::string text(psr_outcome_json(oc, 0, nullptr, 0) + 1, '\0');
  text.resize(psr_outcome_json(oc, 0, &text[0], text.size()));
  psr_outcome_info info{};
  check(psr_outcome_info_get(oc, &info));
  std::vector<psr_confirmed> conf(info.candidates);
  for (uint64_t i = 0; i < info.candidates; ++i)
    check(psr_outcome_candidate(oc, i, &conf[i], nullptr, nullptr));
  psr_outcome_free(oc);
  Value confirmation;
  if (!psrjson::parse(text, confirmation)) throw Fail("internal: outcome JSON");
  const Value *cands = psrjson::field(confirmation, "candidates");
  Value candidates = Value::array(), folded = Value::array();
  for (uint64_t i = 0; i < info.candidates; ++i) {
    const Value &cv = cands->items[i];
    const psr_confirmed &c = conf[i];
    std::printf("#%llu: P=%s ms DM=%s spectral score=%s held-out SNR=%s %s\n",
                (unsigned long long)i, fixed(c.profile.period_s * 1000.0, 6).c_str(),
                fixed(c.refined_dm, 3).c_str(), fixed(c.candidate.score, 2).c_str(),
                fixed(c.validation.snr, 2).c_str(),
                c.accepted ? "ACCEPTED for follow-up" : "REJECTED");
    candidates.push(*psrjson::field(cv, "candidate"));
    Value curve = Value::array();
    for (const Value &p : psrjson::field(cv, "dm_response")->items) {
      Value pt = Value::array();
      pt.push(*psrjson::field(p, "dm"));
      pt.push(*psrjson::field(p, "discovery_profile_response"));
      curve.push(std::move(pt));
    }
    Value f = Value::object();
    f.set("candidate", *psrjson::field(cv, "candidate"));
    f.set("refined_dm", *psrjson::field(cv, "refined_dm"));
    f.set("profile", *psrjson::field(cv, "profile"));
    f.set("dm_curve", std::move(curve));
    f.set("confirmation", cv);
    folded.push(std::move(f));
  }
  Sha256 sha;
  {
    std::ifstream f(a.file, std::ios::binary);
    std::vector<char> buf(1 << 20);
    while (f) {
      f.read(buf.data(), (std::streamsize)buf.size());
      sha.update(reinterpret_cast<const uint8_t *>(buf.data()), (size_t)f.gcount());
    }
  }
  Value revision = Value::null();
  if (FILE *p = popen("git rev-parse HEAD 2>/dev/null", "r")) {
    char buf[128] = {0};
    const bool got = std::fgets(buf, sizeof buf, p) != nullptr;
    if (pclose(p) == 0 && got) {
      std::string r(buf);
      while (!r.empty() && (r.back() == '\n' || r.back() == ' ')) r.pop_back();
      revision = Value::str(r);
    }
  }
  const double elapsed =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
  Value bl = Value::array();
  for (size_t i = 0; i + 1 < birdies.size(); i += 2) {
    Value p = Value::array();
    p.push(Value::num(birdies[i]));
    p.push(Value::num(birdies[i + 1]));
    bl.push(std::move(p));
  }
  Value r = Value::object();
  r.set("schema_version", Value::u64(2));
  r.set("input_sha256", Value::str(sha.hex()));
  r.set("code_revision", revision);
  r.set("confirmation", confirmation);
  r.set("input", Value::str(a.file));
  r.set("version", Value::str("0.1.0"));
  r.set("sample_count", Value::u64(fb.ns));
  r.set("tsamp", Value::num(tsamp));
  r.set("dm_min", Value::num(dm_min));
  r.set("dm_max", Value::num(dm_max));
  r.set("dm_step", Value::num(step));
  r.set("trial_count", Value::u64(nt));
  r.set("common_samples", Value::u64(length));
  r.set("threads", Value::u64(threads));
  r.set("elapsed_seconds", Value::num(elapsed));
  r.set("min_hz", Value::num(min_hz));
  r.set("max_hz", Value::num(max_hz));
  r.set("threshold", Value::num(threshold));
  r.set("birdies", std::move(bl));
  r.set("score_definition",
        Value::str("discovery spectral ranking and approximate profile statistics; "
                   "confirmation fixed-window on/off mean difference / sample standard error "
                   "on disjoint second half; colored noise/RFI may violate independent-noise "
                   "assumptions"));
  r.set("rfi", rfi);
  r.set("candidates", std::move(candidates));
  r.set("folded", std::move(folded));
  write_json(join(out, "report.json"), r);
  std::printf("Saved %s in %ss\n", out.c_str(), fixed(elapsed, 2).c_str());
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  try {
    const Args a = parse_args(argc, argv);
    if (a.cmd == "header") return cmd_header(a);
    if (a.cmd == "fold") return cmd_fold(a);
    if (a.cmd == "dedisperse") return cmd_dedisperse(a);
    if (a.cmd == "inspect") return cmd_inspect(a);
    if (a.cmd == "search") return cmd_search(a);
    if (a.cmd == "synth") return cmd_synth(a);
    throw Fail("unrecognized subcommand '" + a.cmd + "'");
  } catch (const std::exception &e) {
    std::fprintf(stderr, "Error: %s\n", e.what());
    return 1;
  }
}
