// C ABI of libpsr: host-side logic that stays on the host in the reference's
// own terms (header parsing, FP64 delay tables, DM plans, sifting) and the
// entry points that drive the device kernels.
#include <cuda_runtime.h>
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cerrno>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "analyze.h"
#include "psr_internal.h"
#include "refine.h"
#include "search.h"

namespace psr {

namespace {
thread_local std::string g_error;
const double K_DM = 4148.808;  // dedisperse/src/lib.rs:3
}  // namespace

void set_error(const std::string &msg) { g_error = msg; }
const std::string &last_error() { return g_error; }

// ------------------------------------------------------- fbank header
namespace {
bool rd_string(const uint8_t *b, uint64_t len, uint64_t &pos, std::string &out, int &code) {
  if (pos + 4 > len) {
    set_error("failed to fill whole buffer");
    code = PSR_EIO;
    return false;
  }
  int32_t n;
  std::memcpy(&n, b + pos, 4);
  pos += 4;
  if (n < 1 || n > 4096) {
    set_error("invalid or unsupported filterbank: bad string length " + std::to_string(n));
    code = PSR_EFORMAT;
    return false;
  }
  if (pos + (uint64_t)n > len) {
    set_error("failed to fill whole buffer");
    code = PSR_EIO;
    return false;
  }
  out.assign(reinterpret_cast<const char *>(b + pos), (size_t)n);
  pos += (uint64_t)n;
  return true;
}
}  // namespace

// fbank::parse_header (fbank/src/lib.rs:72-147): strict keyword table.
int parse_header_fields(const uint8_t *b, uint64_t len, psr_header &h,
                        psrjson::Value *fields_json);

int parse_header(const uint8_t *b, uint64_t len, psr_header &h) {
  return parse_header_fields(b, len, h, nullptr);
}

int parse_header_fields(const uint8_t *b, uint64_t len, psr_header &h,
                        psrjson::Value *fields_json) {
  static const char *kInts[] = {"machine_id", "telescope_id", "data_type", "barycentric",
                                "pulsarcentric", "nbits", "nsamples", "nchans", "nifs",
                                "nbeams", "ibeam", "signed"};
  static const char *kFloats[] = {"az_start", "za_start", "src_raj", "src_dej", "tstart",
                                  "tsamp", "fch1", "foff", "refdm", "period"};
  struct V {
    int kind;
    int32_t i;
    double f;
    std::string t;
  };
  uint64_t pos = 0;
  int code = PSR_OK;
  std::string s;
  if (!rd_string(b, len, pos, s, code)) return code;
  if (s != "HEADER_START") {
    set_error("invalid or unsupported filterbank: missing HEADER_START");
    return PSR_EFORMAT;
  }
  std::map<std::string, V> f;
  for (;;) {
    std::string key;
    if (!rd_string(b, len, pos, key, code)) return code;
    if (key == "HEADER_END") break;
    V v{};
    if (key == "rawdatafile" || key == "source_name") {
      if (!rd_string(b, len, pos, v.t, code)) return code;
      v.kind = 2;
    } else if (std::any_of(std::begin(kInts), std::end(kInts),
                           [&](const char *k) { return key == k; })) {
      if (pos + 4 > len) {
        set_error("failed to fill whole buffer");
        return PSR_EIO;
      }
      v.kind = 0;
      std::memcpy(&v.i, b + pos, 4);
      pos += 4;
    } else if (std::any_of(std::begin(kFloats), std::end(kFloats),
                           [&](const char *k) { return key == k; })) {
      if (pos + 8 > len) {
        set_error("failed to fill whole buffer");
        return PSR_EIO;
      }
      v.kind = 1;
      std::memcpy(&v.f, b + pos, 8);
      pos += 8;
    } else {
      set_error("invalid or unsupported filterbank: unknown keyword " + key +
                "; cannot infer its type safely");
      return PSR_EFORMAT;
    }
    if (!f.emplace(key, v).second) {
      set_error("invalid or unsupported filterbank: duplicate " + key);
      return PSR_EFORMAT;
    }
  }
  auto geti = [&](const char *k, int32_t &out) {
    auto it = f.find(k);
    if (it == f.end() || it->second.kind != 0) {
      set_error(std::string("invalid or unsupported filterbank: missing integer ") + k);
      return false;
    }
    out = it->second.i;
    return true;
  };
  auto getf = [&](const char *k, double &out) {
    auto it = f.find(k);
    if (it == f.end() || it->second.kind != 1 || !std::isfinite(it->second.f)) {
      set_error(std::string("invalid or unsupported filterbank: missing/invalid float ") + k);
      return false;
    }
    out = it->second.f;
    return true;
  };
  int32_t nchans, nbits;
  double tsamp, fch1, foff;
  if (!geti("nchans", nchans) || !geti("nbits", nbits) || !getf("tsamp", tsamp) ||
      !getf("fch1", fch1) || !getf("foff", foff))
    return PSR_EFORMAT;
  if (nchans <= 0 || tsamp <= 0.0 ||
      !(nbits == 1 || nbits == 2 || nbits == 4 || nbits == 8 || nbits == 16 || nbits == 32)) {
    set_error("invalid or unsupported filterbank: invalid nchans/tsamp/nbits");
    return PSR_EFORMAT;
  }
  auto bad_int = [&](const char *k, int32_t want) {
    auto it = f.find(k);
    return it != f.end() && !(it->second.kind == 0 && it->second.i == want);
  };
  if (bad_int("nifs", 1)) {
    set_error("invalid or unsupported filterbank: only nifs=1 supported");
    return PSR_EFORMAT;
  }
  if (bad_int("signed", 0)) {
    set_error("invalid or unsupported filterbank: signed integer samples unsupported");
    return PSR_EFORMAT;
  }
  if (bad_int("data_type", 1)) {
    set_error("invalid or unsupported filterbank: only filterbank data_type=1 supported");
    return PSR_EFORMAT;
  }
  for (int32_t c = 0; c < nchans; ++c) {
    const double fr = fch1 + (double)c * foff;
    if (!std::isfinite(fr) || fr <= 0.0) {
      set_error("invalid or unsupported filterbank: nonpositive frequency");
      return PSR_EFORMAT;
    }
  }
  h.nchans = nchans;
  h.nbits = nbits;
  h.tsamp = tsamp;
  h.fch1 = fch1;
  h.foff = foff;
  h.data_offset = (int64_t)pos;
  if (fields_json) {
    // fbank::Header as serde writes it: the BTreeMap of keywords (sorted),
    // untagged values, then the parsed scalars (fbank/src/lib.rs:29-38).
    psrjson::Value fm = psrjson::Value::object();
    for (const auto &kv : f) {
      const V &v = kv.second;
      fm.set(kv.first, v.kind == 0   ? psrjson::Value::i64(v.i)
                       : v.kind == 1 ? psrjson::Value::num(v.f)
                                     : psrjson::Value::str(v.t));
    }
    psrjson::Value hv = psrjson::Value::object();
    hv.set("fields", std::move(fm));
    hv.set("nchans", psrjson::Value::u64((uint64_t)nchans));
    hv.set("nbits", psrjson::Value::u64((uint64_t)nbits));
    hv.set("tsamp", psrjson::Value::num(tsamp));
    hv.set("fch1", psrjson::Value::num(fch1));
    hv.set("foff", psrjson::Value::num(foff));
    hv.set("data_offset", psrjson::Value::u64(pos));
    *fields_json = std::move(hv);
  }
  return PSR_OK;
}

// dedisperse::delays (dedisperse/src/lib.rs:9-34); powi(-2) is 1/(f*f).
bool host_delays(const double *f, size_t n, double tsamp, double dm, std::vector<uint64_t> &out) {
  bool bad = n == 0 || !std::isfinite(tsamp) || tsamp <= 0.0 || !std::isfinite(dm) || dm < 0.0;
  for (size_t i = 0; i < n && !bad; ++i) bad = !std::isfinite(f[i]) || f[i] <= 0.0;
  if (bad) {
    set_error(
        "invalid dedispersion input: positive frequencies/tsamp and nonnegative DM required");
    return false;
  }
  double ref = 0.0;
  for (size_t i = 0; i < n; ++i) ref = std::fmax(ref, f[i]);
  const double rinv = 1.0 / (ref * ref);
  out.resize(n);
  for (size_t i = 0; i < n; ++i) {
    const double s = std::round(K_DM * dm * (1.0 / (f[i] * f[i]) - rinv) / tsamp);
    if (s > 18446744073709551615.0) {
      set_error("invalid dedispersion input: delay overflow");
      return false;
    }
    out[i] = s > 0.0 ? (uint64_t)s : 0;
  }
  return true;
}

namespace {

struct Stream {
  cudaStream_t s = nullptr;
  Stream() { cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking); }
  ~Stream() {
    if (s) cudaStreamDestroy(s);
  }
};

// Decode the header and stage the payload on the device (fbank/src/lib.rs:149-170).
int obs_from_bytes(const uint8_t *bytes, uint64_t len, int64_t limit, DeviceObs &o,
                   cudaStream_t st) {
  PSR_TRY(parse_header(bytes, len, o.h));
  const uint64_t plen = len - (uint64_t)o.h.data_offset;
  const uint64_t bpf = (uint64_t)o.h.nchans * (uint64_t)o.h.nbits;
  const uint64_t bits = plen * 8;
  if (bits % bpf != 0) {
    set_error("invalid or unsupported filterbank: truncated frame or packed padding unsupported");
    return PSR_EFORMAT;
  }
  const uint64_t total = bits / bpf;
  const uint64_t ns = limit < 0 ? total : std::min<uint64_t>((uint64_t)limit, total);
  if (ns < 2) {
    set_error("invalid or unsupported filterbank: need at least two samples");
    return PSR_EFORMAT;
  }
  o.ns = ns;
  o.nch = (uint64_t)o.h.nchans;
  o.kind = kind_for_bits(o.h.nbits);
  o.payload_bytes = (ns * bpf + 7) / 8;
  PSR_TRY(o.payload.ensure(o.payload_bytes + 16));
  PSR_CUDA(cudaMemcpyAsync(o.payload.p, bytes + o.h.data_offset, o.payload_bytes,
                           cudaMemcpyHostToDevice, st));
  PSR_TRY(o.alloc(st));
  return PSR_OK;
}

int unpack_checked(DeviceObs &o, DevBuf &errbuf, cudaStream_t st) {
  PSR_TRY(errbuf.ensure(8));
  PSR_CUDA(cudaMemsetAsync(errbuf.p, 0xff, 8, st));
  PSR_TRY(launch_unpack(o, errbuf.as<unsigned long long>(), st));
  unsigned long long e = 0;
  PSR_CUDA(cudaMemcpyAsync(&e, errbuf.p, 8, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  if (e != ~0ull) {
    set_error("invalid or unsupported filterbank: nonfinite sample at " +
              std::to_string(e / o.nch) + "/" + std::to_string(e % o.nch));
    return PSR_EFORMAT;
  }
  return PSR_OK;
}

bool valid_config(const psr_search_config *c) {
  return c && c->max_candidates >= 1 && c->max_candidates <= 64 && !std::isnan(c->min_hz) &&
         !std::isnan(c->max_hz) && !std::isnan(c->threshold) && (c->nbirdies == 0 || c->birdies) &&
         (c->max_harmonics == 0 || c->max_harmonics == 16 || c->max_harmonics == 32);
}

SpecConfig to_spec(const psr_search_config *c, double tsamp) {
  SpecConfig s;
  s.tsamp = tsamp;
  s.min_hz = c->min_hz;
  s.max_hz = c->max_hz;
  s.threshold = c->threshold;
  s.max_candidates = c->max_candidates;
  s.birdies.assign(c->birdies, c->birdies + 2 * c->nbirdies);
  s.levels = c->max_harmonics == 32 ? 6 : 5;
  return s;
}

// A filterbank made from a host f32 array (channel-major), for the entry
// points that take host series or arrays.
int obs_from_f32(const float *data, uint64_t nch, uint64_t ns, double tsamp, DeviceObs &o,
                 cudaStream_t st) {
  o.h = psr_header{(int64_t)nch, 32, tsamp, 1.0, 0.0, 0};
  o.ns = ns;
  o.nch = nch;
  o.kind = SAMPLE_F32;
  PSR_TRY(o.alloc(st));
  PSR_CUDA(cudaMemcpy2DAsync(o.samples.p, o.ld * 4, data, ns * 4, ns * 4, nch,
                             cudaMemcpyHostToDevice, st));
  return PSR_OK;
}

}  // namespace
}  // namespace psr

using namespace psr;

struct psr_fb {
  DeviceObs o;
  Stream stream;
};

struct psr_session {
  DeviceObs o;
  Stream stream;
  RfiWork rfi;
  RfiResult rfi_res;
  uint64_t rfi_block = 0;
  float rfi_threshold = 8.0f;
  SearchEngine eng;
  std::vector<double> trials;
  uint64_t discovery = 0;
  SpecConfig spec;
  DevBuf errbuf;
  HostBuf h_err;  // sync()'s copy of errbuf
  bool have_run = false;
  // unpack / rfi timing (the engine times its own stages)
  std::vector<cudaEvent_t> ev[2][2];
  double pre_ms[2] = {0, 0};
  uint64_t pre_launches[2] = {0, 0};
  int mark(int stage, int which) {
    if (!eng.profile) return PSR_OK;
    cudaEvent_t e;
    PSR_CUDA(cudaEventCreate(&e));
    PSR_CUDA(cudaEventRecord(e, stream.s));
    ev[stage][which].push_back(e);
    if (which) pre_launches[stage] += 1;
    return PSR_OK;
  }
  int harvest() {
    for (int st = 0; st < 2; ++st) {
      for (size_t i = 0; i < ev[st][0].size() && i < ev[st][1].size(); ++i) {
        float ms = 0.0f;
        PSR_CUDA(cudaEventElapsedTime(&ms, ev[st][0][i], ev[st][1][i]));
        pre_ms[st] += ms;
      }
      for (int w = 0; w < 2; ++w) {
        for (cudaEvent_t e : ev[st][w]) cudaEventDestroy(e);
        ev[st][w].clear();
      }
    }
    return PSR_OK;
  }
  ~psr_session() {
    for (int st = 0; st < 2; ++st)
      for (int w = 0; w < 2; ++w)
        for (cudaEvent_t e : ev[st][w]) cudaEventDestroy(e);
  }
};

namespace psr {
template <class T>
__global__ void k_to_f32(const T *s, uint64_t ld, uint64_t ns, uint64_t nch, float *out) {
  const uint64_t id = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= ns * nch) return;
  const uint64_t c = id / ns, t = id % ns;
  out[id] = (float)s[c * ld + t];
}

}  // namespace psr

extern "C" {

const char *psr_version(void) { return "pulsarsr-gb300 0.1.0 sm_103a"; }

uint64_t psr_last_error(char *buf, uint64_t len) {
  const std::string &e = last_error();
  if (buf && len) {
    const uint64_t n = std::min<uint64_t>(len - 1, e.size());
    std::memcpy(buf, e.data(), n);
    buf[n] = 0;
  }
  return e.size();
}

int psr_header_json(const uint8_t *bytes, uint64_t len, int pretty, char *buf, uint64_t cap,
                    uint64_t *needed) {
  if (!bytes || !needed) {
    set_error("header_json: null argument");
    return PSR_EINVAL;
  }
  psr_header h;
  psrjson::Value v;
  PSR_TRY(parse_header_fields(bytes, len, h, &v));
  const std::string s = psrjson::dump(v, pretty != 0);
  *needed = s.size();
  if (buf && cap) {
    const uint64_t n = std::min<uint64_t>(cap - 1, s.size());
    std::memcpy(buf, s.data(), n);
    buf[n] = '\0';
  }
  return PSR_OK;
}

int psr_parse_header(const uint8_t *bytes, uint64_t len, psr_header *out) {
  if (!bytes || !out) {
    set_error("parse_header: null argument");
    return PSR_EINVAL;
  }
  return parse_header(bytes, len, *out);
}

int psr_fb_decode(const uint8_t *bytes, uint64_t len, int64_t limit, psr_fb **out) {
  if (!bytes || !out) {
    set_error("decode: null argument");
    return PSR_EINVAL;
  }
  std::unique_ptr<psr_fb> fb(new psr_fb());
  PSR_TRY(obs_from_bytes(bytes, len, limit, fb->o, fb->stream.s));
  DevBuf e;
  PSR_TRY(unpack_checked(fb->o, e, fb->stream.s));
  *out = fb.release();
  return PSR_OK;
}

// fbank::read (fbank/src/lib.rs:198-203): the header is parsed from the
// file's first bytes, then the payload streams to the device through two
// pinned staging buffers (the read of one chunk overlaps the copy of the
// previous one) and is unpacked there; the file is never held whole in host
// memory.
int psr_fb_read(const char *path, int64_t limit, psr_fb **out) {
  if (!path || !out) {
    set_error("read: null argument");
    return PSR_EINVAL;
  }
  const int fd = open(path, O_RDONLY);
  if (fd < 0) {
    set_error(std::string(std::strerror(errno)) + " (os error " + std::to_string(errno) + ")");
    return PSR_EIO;
  }
  struct Closer {
    int fd;
    ~Closer() { close(fd); }
  } closer{fd};
  struct stat stt;
  if (fstat(fd, &stt) != 0) {
    set_error(std::string(std::strerror(errno)));
    return PSR_EIO;
  }
  const uint64_t fsize = (uint64_t)stt.st_size;
  auto read_at = [&](uint8_t *dst, uint64_t n, uint64_t off) -> bool {
    uint64_t done = 0;
    while (done < n) {
      const ssize_t r = pread(fd, dst + done, n - done, (off_t)(off + done));
      if (r <= 0) return false;
      done += (uint64_t)r;
    }
    return true;
  };
  // Header: SIGPROC headers are a few hundred bytes; 64 KiB bounds them.
  std::vector<uint8_t> head((size_t)std::min<uint64_t>(fsize, 65536));
  if (!read_at(head.data(), head.size(), 0)) {
    set_error("failed to fill whole buffer");
    return PSR_EIO;
  }
  std::unique_ptr<psr_fb> fb(new psr_fb());
  DeviceObs &o = fb->o;
  PSR_TRY(parse_header(head.data(), head.size(), o.h));
  const uint64_t plen = fsize - (uint64_t)o.h.data_offset;
  const uint64_t bpf = (uint64_t)o.h.nchans * (uint64_t)o.h.nbits;
  if ((plen * 8) % bpf != 0) {
    set_error("invalid or unsupported filterbank: truncated frame or packed padding unsupported");
    return PSR_EFORMAT;
  }
  const uint64_t total = plen * 8 / bpf;
  const uint64_t ns = limit < 0 ? total : std::min<uint64_t>((uint64_t)limit, total);
  if (ns < 2) {
    set_error("invalid or unsupported filterbank: need at least two samples");
    return PSR_EFORMAT;
  }
  o.ns = ns;
  o.nch = (uint64_t)o.h.nchans;
  o.kind = kind_for_bits(o.h.nbits);
  o.payload_bytes = (ns * bpf + 7) / 8;
  PSR_TRY(o.payload.ensure(o.payload_bytes + 16));
  cudaStream_t st = fb->stream.s;
  PSR_TRY(o.alloc(st));
  constexpr uint64_t CHUNK = 64ull << 20;
  uint8_t *stage[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  struct Staging {
    uint8_t **b;
    cudaEvent_t *e;
    ~Staging() {
      for (int i = 0; i < 2; ++i) {
        if (e[i]) {
          cudaEventSynchronize(e[i]);
          cudaEventDestroy(e[i]);
        }
        if (b[i]) cudaFreeHost(b[i]);
      }
    }
  } staging{stage, done};
  for (int i = 0; i < 2; ++i) {
    PSR_CUDA(cudaHostAlloc((void **)&stage[i], CHUNK, cudaHostAllocDefault));
    PSR_CUDA(cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming));
  }
  uint64_t off = 0;
  for (int i = 0; off < o.payload_bytes; ++i, off += CHUNK) {
    const int k = i & 1;
    const uint64_t n = std::min(CHUNK, o.payload_bytes - off);
    PSR_CUDA(cudaEventSynchronize(done[k]));  // the copy that last used stage[k]
    if (!read_at(stage[k], n, (uint64_t)o.h.data_offset + off)) {
      set_error("failed to fill whole buffer");
      return PSR_EIO;
    }
    PSR_CUDA(cudaMemcpyAsync(o.payload.as<uint8_t>() + off, stage[k], n, cudaMemcpyHostToDevice,
                             st));
    PSR_CUDA(cudaEventRecord(done[k], st));
  }
  DevBuf e;
  PSR_TRY(unpack_checked(o, e, st));
  *out = fb.release();
  return PSR_OK;
}

int psr_fb_synth(const psr_synth_config *cfg, psr_fb **out) {
  if (!cfg || !out) {
    set_error("invalid synthetic configuration");
    return PSR_EINVAL;
  }
  std::unique_ptr<psr_fb> fb(new psr_fb());
  PSR_TRY(synth_obs(*cfg, fb->o, fb->stream.s));
  *out = fb.release();
  return PSR_OK;
}

int psr_fb_inject_rfi(psr_fb *fb, const psr_synth_rfi *rfi) {
  if (!fb || !rfi) {
    set_error("invalid interference configuration");
    return PSR_EINVAL;
  }
  return inject_rfi(fb->o, *rfi, fb->stream.s);
}

int psr_fb_info(const psr_fb *fb, psr_header *header, uint64_t *nsamples) {
  if (!fb) {
    set_error("fb_info: null handle");
    return PSR_EINVAL;
  }
  if (header) *header = fb->o.h;
  if (nsamples) *nsamples = fb->o.ns;
  return PSR_OK;
}

int psr_fb_download_channels(const psr_fb *fb, uint64_t c0, uint64_t nchannels, float *out) {
  if (!fb || !out || c0 > fb->o.nch || nchannels > fb->o.nch - c0) {
    set_error("fb_download: null argument or channel range outside the filterbank");
    return PSR_EINVAL;
  }
  const DeviceObs &o = fb->o;
  if (nchannels == 0) return PSR_OK;
  cudaStream_t st = fb->stream.s;
  DevBuf tmp;
  PSR_TRY(tmp.ensure(o.ns * nchannels * 4));
  const unsigned g = (unsigned)((o.ns * nchannels + 255) / 256);
  switch (o.kind) {
    case SAMPLE_U8: k_to_f32<uint8_t><<<g, 256, 0, st>>>(o.samples.as<uint8_t>() + c0 * o.ld, o.ld, o.ns, nchannels, tmp.as<float>()); break;
    case SAMPLE_U16: k_to_f32<uint16_t><<<g, 256, 0, st>>>(o.samples.as<uint16_t>() + c0 * o.ld, o.ld, o.ns, nchannels, tmp.as<float>()); break;
    default: k_to_f32<float><<<g, 256, 0, st>>>(o.samples.as<float>() + c0 * o.ld, o.ld, o.ns, nchannels, tmp.as<float>());
  }
  PSR_CUDA(cudaGetLastError());
  PSR_CUDA(cudaMemcpyAsync(out, tmp.p, o.ns * nchannels * 4, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  return PSR_OK;
}

int psr_fb_download(const psr_fb *fb, float *out) {
  if (!fb || !out) {
    set_error("fb_download: null argument");
    return PSR_EINVAL;
  }
  return psr_fb_download_channels(fb, 0, fb->o.nch, out);
}

void psr_fb_free(psr_fb *fb) { delete fb; }

int psr_median(const float *values, uint64_t n, float *out) {
  if (!out || (n && !values)) {
    set_error("median: null argument");
    return PSR_EINVAL;
  }
  Stream s;
  DevBuf v, r;
  PSR_TRY(v.ensure(std::max<uint64_t>(n, 1) * 4));
  PSR_TRY(r.ensure(4));
  if (n) PSR_CUDA(cudaMemcpyAsync(v.p, values, n * 4, cudaMemcpyHostToDevice, s.s));
  PSR_TRY(launch_median_f32(v.as<float>(), n, r.as<float>(), nullptr, s.s));
  PSR_CUDA(cudaMemcpyAsync(out, r.p, 4, cudaMemcpyDeviceToHost, s.s));
  PSR_CUDA(cudaStreamSynchronize(s.s));
  return PSR_OK;
}

int psr_rfi_mask(psr_fb *fb, uint64_t block_samples, float threshold, uint64_t *channels,
                 uint64_t *nchannels_bad, uint64_t *blocks, uint64_t blocks_cap,
                 uint64_t *nblocks_bad, double *masked_fraction) {
  if (!fb || !nchannels_bad || !nblocks_bad || !masked_fraction) {
    set_error("rfi::mask: null argument");
    return PSR_EINVAL;
  }
  RfiWork w;
  RfiResult res;
  PSR_TRY(rfi_enqueue(fb->o, block_samples, threshold, w, fb->stream.s));
  PSR_TRY(rfi_collect(fb->o, block_samples, w, fb->stream.s, res));
  *nchannels_bad = res.channels.size();
  if (channels) std::copy(res.channels.begin(), res.channels.end(), channels);
  *nblocks_bad = res.blocks.size();
  if (blocks)
    for (uint64_t i = 0; i < res.blocks.size() && i < blocks_cap; ++i) blocks[i] = res.blocks[i];
  *masked_fraction = res.masked_fraction;
  if (res.blocks.size() > blocks_cap && blocks) {
    set_error("rfi::mask: blocks buffer too small");
    return PSR_ECAPACITY;
  }
  return PSR_OK;
}

int psr_channel_stats(const psr_fb *fb, float *means, float *variances) {
  if (!fb || !means || !variances) {
    set_error("channel_stats: null argument");
    return PSR_EINVAL;
  }
  return rfi_channel_stats(fb->o, means, variances, fb->stream.s);
}

int psr_delays(const double *freqs, uint64_t nchans, double tsamp, double dm, uint64_t *out) {
  std::vector<uint64_t> d;
  if (!host_delays(freqs, nchans, tsamp, dm, d)) return PSR_EDEDISPERSE;
  std::copy(d.begin(), d.end(), out);
  return PSR_OK;
}

int psr_dm_step(const double *f, uint64_t n, double tsamp, double *out) {
  std::vector<uint64_t> tmp;
  if (!host_delays(f, n, tsamp, 0.0, tmp)) return PSR_EDEDISPERSE;
  double lo = INFINITY, hi = 0.0;
  for (uint64_t i = 0; i < n; ++i) {
    lo = std::fmin(lo, f[i]);
    hi = std::fmax(hi, f[i]);
  }
  const double span = K_DM * (1.0 / (lo * lo) - 1.0 / (hi * hi));
  if (span <= 0.0) {
    set_error("invalid dedispersion input: DM planning requires finite bandwidth");
    return PSR_EDEDISPERSE;
  }
  *out = tsamp / span;
  return PSR_OK;
}

int psr_plan(double mn, double mx, double step, double *out, uint64_t cap, uint64_t *n) {
  if (!std::isfinite(mn) || !std::isfinite(mx) || !std::isfinite(step) || mn < 0.0 || mx < mn ||
      step <= 0.0) {
    set_error("invalid dedispersion input: invalid DM bounds/step");
    return PSR_EDEDISPERSE;
  }
  const uint64_t cnt = (uint64_t)std::floor((mx - mn) / step) + 1;
  if (cnt > 100000) {
    set_error("invalid dedispersion input: more than 100000 DM trials");
    return PSR_EDEDISPERSE;
  }
  *n = cnt;
  if (out && cap < cnt) {
    set_error("plan: output buffer too small");
    return PSR_ECAPACITY;
  }
  if (out)
    for (uint64_t i = 0; i < cnt; ++i) out[i] = mn + (double)i * step;
  return PSR_OK;
}

namespace {
uint64_t series_ld_(uint64_t n) { return series_ld(n); }

// Dedisperse with explicit per-channel delays (one trial) on a device obs.
int dedisperse_delays(const DeviceObs &o, const uint64_t *d, int64_t length, float *out,
                      uint64_t cap, uint64_t *n_out, cudaStream_t st) {
  uint64_t maxd = 0;
  for (uint64_t c = 0; c < o.nch; ++c) maxd = std::max(maxd, d[c]);
  if (maxd > o.ns) {
    set_error("invalid dedispersion input: delay exceeds observation");
    return PSR_EDEDISPERSE;
  }
  const uint64_t avail = o.ns - maxd;
  const uint64_t n = length < 0 ? avail : (uint64_t)length;
  if (n < 2 || n > avail) {
    set_error("invalid dedispersion input: invalid output length");
    return PSR_EDEDISPERSE;
  }
  *n_out = n;
  if (!out) return PSR_OK;
  if (cap < n) {
    set_error("dedisperse: output buffer too small");
    return PSR_ECAPACITY;
  }
  std::vector<uint32_t> tab(o.nch);
  for (uint64_t c = 0; c < o.nch; ++c) tab[c] = (uint32_t)d[c];
  uint64_t spread = 0;
  DevBuf dd, ser, parts, sums, means, err;
  PSR_TRY(dd.ensure(o.nch * 4));
  PSR_CUDA(cudaMemcpyAsync(dd.p, tab.data(), o.nch * 4, cudaMemcpyHostToDevice, st));
  const uint64_t ldo = series_ld_(n);
  PSR_TRY(ser.ensure(ldo * 4 + 256));
  PSR_TRY(parts.ensure(dedisperse_part_count(o, n) * 8 + 8));
  PSR_TRY(sums.ensure(8));
  PSR_TRY(means.ensure(8));
  PSR_TRY(err.ensure(8));
  PSR_CUDA(cudaMemsetAsync(err.p, 0, 8, st));
  PSR_TRY(launch_dedisperse_ex(o, dd.as<uint32_t>(), 1, n, ser.as<float>(), ldo,
                               parts.as<double>(), sums.as<double>(), means.as<float>(), spread,
                               err.as<unsigned>(), st, 0, 0, false));
  PSR_CUDA(cudaMemcpyAsync(out, ser.p, n * 4, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  return PSR_OK;
}
}  // namespace

int psr_dedisperse(const psr_fb *fb, const uint64_t *delays, int64_t length, float *out,
                   uint64_t cap, uint64_t *n_out) {
  if (!fb || !delays || !n_out) {
    set_error("invalid dedispersion input: array shape mismatch");
    return PSR_EDEDISPERSE;
  }
  return dedisperse_delays(fb->o, delays, length, out, cap, n_out, fb->stream.s);
}

int psr_dedisperse_trials(const psr_fb *fb, const double *trials, uint64_t ntrials,
                          uint64_t length, float *out, double *sums_out) {
  if (!fb || !trials || !out || ntrials == 0) {
    set_error("dedisperse_trials: null argument or empty plan");
    return PSR_EINVAL;
  }
  const DeviceObs &o = fb->o;
  cudaStream_t st = fb->stream.s;
  std::vector<uint32_t> tab;
  uint64_t spread = 0, maxd = 0;
  PSR_TRY(make_delay_table(o, trials, ntrials, tab, spread, maxd));
  if (length < 2 || length > o.ns - maxd) {
    set_error("invalid dedispersion input: invalid output length");
    return PSR_EDEDISPERSE;
  }
  const uint64_t ldo = series_ld(length);
  DevBuf dd, ser, parts, sums, means, err;
  PSR_TRY(dd.ensure(tab.size() * 4));
  PSR_CUDA(cudaMemcpyAsync(dd.p, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice, st));
  PSR_TRY(ser.ensure(ntrials * ldo * 4 + 256));
  PSR_TRY(parts.ensure(ntrials * dedisperse_part_count(o, length) * 8 + 8));
  PSR_TRY(sums.ensure(ntrials * 8));
  PSR_TRY(means.ensure(ntrials * 4));
  PSR_TRY(err.ensure(8));
  PSR_CUDA(cudaMemsetAsync(err.p, 0, 8, st));
  SubbandPlan sbp;
  const int G = o.kind == SAMPLE_U8 ? dedisp_subbands_default(o) : 0;
  PSR_TRY(build_subband_plan(tab, o.nch, {0, ntrials}, G, sbp, st));
  PSR_TRY(launch_dedisperse_ex(o, dd.as<uint32_t>(), ntrials, length, ser.as<float>(), ldo,
                               parts.as<double>(), sums.as<double>(), means.as<float>(), spread,
                               err.as<unsigned>(), st, 0, 0, sums_out != nullptr, &sbp, 0));
  PSR_CUDA(cudaMemcpy2DAsync(out, length * 4, ser.p, ldo * 4, length * 4, ntrials,
                             cudaMemcpyDeviceToHost, st));
  if (sums_out)
    PSR_CUDA(cudaMemcpyAsync(sums_out, sums.p, ntrials * 8, cudaMemcpyDeviceToHost, st));
  unsigned e = 0;
  PSR_CUDA(cudaMemcpyAsync(&e, err.p, 4, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  if (e) {
    set_error("dedispersion: a bounded wait for a staged tile gave up");
    return PSR_ETIMEOUT;
  }
  return PSR_OK;
}

int psr_test_stage_timeout(const psr_fb *fb, uint64_t spin_limit) {
  if (!fb || spin_limit == 0 || spin_limit > (1ull << 26)) {
    set_error("test_stage_timeout: a filterbank and a spin limit in [1, 2^26] are required");
    return PSR_EINVAL;
  }
  const DeviceObs &o = fb->o;
  cudaStream_t st = fb->stream.s;
  const uint64_t n = std::min<uint64_t>(o.ns, 8192);
  std::vector<uint32_t> tab(o.nch, 0);
  DevBuf dd, ser, parts, sums, means, err;
  PSR_TRY(dd.ensure(o.nch * 4));
  PSR_CUDA(cudaMemcpyAsync(dd.p, tab.data(), o.nch * 4, cudaMemcpyHostToDevice, st));
  const uint64_t ldo = series_ld(n);
  PSR_TRY(ser.ensure(ldo * 4 + 256));
  PSR_TRY(parts.ensure(dedisperse_part_count(o, n) * 8 + 8));
  PSR_TRY(sums.ensure(8));
  PSR_TRY(means.ensure(8));
  PSR_TRY(err.ensure(8));
  PSR_CUDA(cudaMemsetAsync(err.p, 0, 8, st));
  PSR_TRY(launch_dedisperse_ex(o, dd.as<uint32_t>(), 1, n, ser.as<float>(), ldo,
                               parts.as<double>(), sums.as<double>(), means.as<float>(), 0,
                               err.as<unsigned>(), st, (long long)spin_limit, 1));
  unsigned e = 0;
  PSR_CUDA(cudaMemcpyAsync(&e, err.p, 4, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  if (!e) {
    set_error("test_stage_timeout: this filterbank does not take the staged kernel");
    return PSR_EINVAL;
  }
  set_error("dedispersion: a bounded wait for a staged tile gave up");
  return PSR_ETIMEOUT;
}

int psr_raw_power(const float *series, uint64_t len, float *out) {
  if (!series || !out || len < 2) {
    set_error("periodicity: series of at least two samples required");
    return PSR_EINVAL;
  }
  Stream s;
  FftPlan p;
  PSR_TRY(p.init(len, s.s));
  const uint64_t ldo = series_ld_(len);
  DevBuf ser, sums, work, power, psum;
  PSR_TRY(ser.ensure(ldo * 4 + 256));
  PSR_TRY(sums.ensure(8));
  PSR_TRY(work.ensure(p.M * 8 + 16));
  PSR_TRY(power.ensure((p.M + 1 + 64) * 4));
  PSR_TRY(psum.ensure(p.pass2_ctas() * 8 + 8));
  PSR_CUDA(cudaMemcpyAsync(ser.p, series, len * 4, cudaMemcpyHostToDevice, s.s));
  PSR_TRY(launch_series_mean(ser.as<float>(), len, nullptr, sums.as<float>(), s.s));
  PSR_TRY(launch_raw_power_ex(p, ser.as<float>(), ldo, sums.as<float>(), 1, work.as<float2>(),
                              power.as<float>(), ((p.M + 1 + 63) / 64) * 64, psum.as<double>(),
                              s.s));
  PSR_CUDA(cudaMemcpyAsync(out, power.p, (p.M + 1) * 4, cudaMemcpyDeviceToHost, s.s));
  PSR_CUDA(cudaStreamSynchronize(s.s));
  return PSR_OK;
}

int psr_periodicity(const float *series, uint64_t len, double tsamp, double dm,
                    const psr_search_config *cfg, psr_candidate *out, uint64_t cap,
                    uint64_t *n) {
  if (!series || len < 2 || !std::isfinite(tsamp) || tsamp <= 0.0 || !valid_config(cfg) || !n) {
    set_error("periodicity: series.len() >= 2, finite positive tsamp and a valid config "
              "are required");
    return PSR_EINVAL;
  }
  // A one-channel f32 filterbank with zero delay reproduces the series.
  Stream s;
  DeviceObs o;
  PSR_TRY(obs_from_f32(series, 1, len, tsamp, o, s.s));
  SearchEngine e;
  e.chunk = 1;
  PSR_TRY(e.prepare(o, &dm, 1, len, to_spec(cfg, tsamp), s.s));
  // The engine computes delays from the DM; with one channel they are zero.
  PSR_TRY(e.enqueue(o, s.s));
  PSR_TRY(e.finish(o, s.s));
  uint64_t counts = 0;
  return e.collect(s.s, &counts, out, cap, n);
}

int psr_search_trials(const psr_fb *fb, const double *trials, uint64_t ntrials,
                      uint64_t discovery, const psr_search_config *cfg, uint64_t *counts,
                      psr_candidate *out, uint64_t cap, uint64_t *n_total) {
  if (!fb || !trials || !valid_config(cfg) || !n_total) {
    set_error("search: null argument or invalid config");
    return PSR_EINVAL;
  }
  cudaStream_t st = fb->stream.s;
  SearchEngine e;
  PSR_TRY(e.prepare(fb->o, trials, ntrials, discovery, to_spec(cfg, fb->o.h.tsamp), st));
  PSR_TRY(e.enqueue(fb->o, st));
  PSR_TRY(e.finish(fb->o, st));
  return e.collect(st, counts, out, cap, n_total);
}

int psr_analyze(const psr_fb *fb, const double *trials, uint64_t ntrials,
                const psr_candidate *generated, uint64_t ngenerated, uint64_t limit,
                uint64_t bins, const psr_rules *rules, psr_outcome **out) {
  if (!fb || !out || (!generated && ngenerated)) {
    set_error("analyze: null argument");
    return PSR_EINVAL;
  }
  psr_rules r;
  psr_rules_default(&r);
  std::unique_ptr<psr_outcome> o(new psr_outcome());
  PSR_TRY(analyze_obs(fb->o, trials, ntrials, generated, ngenerated, limit, bins,
                      rules ? *rules : r, o->o, fb->stream.s));
  *out = o.release();
  return PSR_OK;
}

// ------------------------------------------------ gradient refinement
namespace {
int refine_options(const psr_refine_options *o, RefineOptions &r) {
  if (o) {
    r.bins = o->bins;
    r.subints = o->subints;
    r.max_evals = o->max_evals;
    r.tol = o->tol_bins;
    r.exact = o->exact != 0;
    r.dm_window = o->dm_window;
  }
  if (r.bins < 4 || r.subints < 1 || r.max_evals < 1 || !(r.tol > 0.0)) {
    set_error("refine: bins >= 4, subints >= 1, max_evals >= 1 and tol_bins > 0 required");
    return PSR_EINVAL;
  }
  return PSR_OK;
}
int refine_length(const psr_fb *fb, uint64_t n) {
  if (!fb || n < 16 || n + 2 > fb->o.ns) {
    set_error("refine: 16 <= n <= nsamples - 2 required");
    return PSR_EINVAL;
  }
  return PSR_OK;
}
}  // namespace

int psr_refine_objective(const psr_fb *fb, uint64_t n, const psr_timing *theta,
                         const psr_refine_options *opt, double variance, double *J, double *grad,
                         double *profile, double *subint_profiles) {
  PSR_TRY(refine_length(fb, n));
  RefineOptions ro;
  PSR_TRY(refine_options(opt, ro));
  if (!theta || !J) {
    set_error("refine: null argument");
    return PSR_EINVAL;
  }
  RefineWork w;
  RefineEval ev;
  PSR_TRY(w.evaluate(fb->o, n, *theta, ro, 1.0, ev, fb->stream.s));
  const double v = variance > 0.0 ? variance : (ev.var_y > 0.0 ? ev.var_y : 1.0);
  *J = ev.J / v;
  if (grad) {
    grad[0] = ev.dP / v;
    grad[1] = ev.dPdot / v;
    grad[2] = ev.dDM / v;
  }
  if (profile) std::copy(ev.profile.begin(), ev.profile.end(), profile);
  if (subint_profiles) std::copy(ev.cells.begin(), ev.cells.end(), subint_profiles);
  return PSR_OK;
}

int psr_refine_cube_objective(const psr_fb *fb, uint64_t n, const psr_timing *reference,
                              const psr_timing *theta, uint64_t npoints,
                              const psr_refine_options *opt, double *J, double *grad) {
  PSR_TRY(refine_length(fb, n));
  RefineOptions ro;
  PSR_TRY(refine_options(opt, ro));
  if (!reference || !theta || !J || npoints == 0) {
    set_error("refine: null argument");
    return PSR_EINVAL;
  }
  std::vector<double> g(3 * npoints);
  PSR_TRY(cube_objective(fb->o, n, *reference, theta, npoints, ro, J, g.data(), fb->stream.s));
  if (grad) {
    // (nu, nudot) = (1/P, -Pdot/P^2): the chain rule to (P, Pdot).
    for (uint64_t k = 0; k < npoints; ++k) {
      const double P = theta[k].period_s, Pd = theta[k].pdot;
      const double gnu = g[3 * k], gnd = g[3 * k + 1];
      grad[3 * k] = gnu * (-1.0 / (P * P)) + gnd * (2.0 * Pd / (P * P * P));
      grad[3 * k + 1] = gnd * (-1.0 / (P * P));
      grad[3 * k + 2] = g[3 * k + 2];
    }
  }
  return PSR_OK;
}

int psr_refine_gradient(const psr_fb *fb, uint64_t n, const psr_timing *start, uint64_t ncand,
                        const psr_refine_options *opt, psr_timing *out, double *J,
                        uint64_t *evals) {
  PSR_TRY(refine_length(fb, n));
  RefineOptions ro;
  PSR_TRY(refine_options(opt, ro));
  if ((!start || !out) && ncand) {
    set_error("refine: null argument");
    return PSR_EINVAL;
  }
  if (ro.exact) {
    RefineWork w;
    for (uint64_t i = 0; i < ncand; ++i) {
      double j = 0.0;
      uint64_t e = 0;
      PSR_TRY(refine_gradient_one(fb->o, n, start[i], ro, w, out[i], j, e, fb->stream.s));
      if (J) J[i] = j;
      if (evals) evals[i] = e;
    }
    return PSR_OK;
  }
  for (uint64_t i = 0; i < ncand; ++i)
    if (!(start[i].period_s > 0.0) || !std::isfinite(start[i].period_s) ||
        !std::isfinite(start[i].pdot) || !(start[i].dm >= 0.0)) {
      set_error("refine: finite positive period, finite pdot and nonnegative DM required");
      return PSR_EINVAL;
    }
  // Group nearby starting points (sorted by DM, then frequency): at most 16
  // per cube, within half a cycle of frequency drift over the observation and
  // a quarter cycle of DM smear across the band of the group's first member.
  const DeviceObs &o = fb->o;
  double fmax = 0.0, fmin = 1e300;
  for (uint64_t c = 0; c < o.nch; ++c) {
    const double f = o.h.fch1 + (double)c * o.h.foff;
    fmax = std::fmax(fmax, f);
    fmin = std::fmin(fmin, f);
  }
  const double kspan = 4148.808 * (1.0 / (fmin * fmin) - 1.0 / (fmax * fmax));
  const double T = (double)n * o.h.tsamp;
  std::vector<uint64_t> idx(ncand);
  for (uint64_t i = 0; i < ncand; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) {
    if (start[a].dm != start[b].dm) return start[a].dm < start[b].dm;
    return start[a].period_s > start[b].period_s;
  });
  std::vector<uint64_t> pending = idx;
  CubeCache cache;
  while (!pending.empty()) {
    const uint64_t lead = pending.front();
    const double nu0 = 1.0 / start[lead].period_s;
    std::vector<uint64_t> group, rest;
    for (uint64_t k : pending) {
      const double nu = 1.0 / start[k].period_s;
      const bool near = std::fabs(nu - nu0) * T <= 0.5 &&
                        std::fabs(start[k].dm - start[lead].dm) * kspan * nu0 <= 0.25 &&
                        std::fabs(start[k].pdot - start[lead].pdot) * nu0 * nu0 * T * T <= 1.0;
      if (near && group.size() < 16) group.push_back(k);
      else rest.push_back(k);
    }
    std::vector<psr_timing> gs(group.size()), go(group.size());
    std::vector<double> gj(group.size());
    std::vector<uint64_t> ge(group.size());
    for (size_t i = 0; i < group.size(); ++i) gs[i] = start[group[i]];
    PSR_TRY(refine_cube_group(o, n, gs.data(), group.size(), ro, go.data(), gj.data(),
                              ge.data(), cache, fb->stream.s));
    for (size_t i = 0; i < group.size(); ++i) {
      out[group[i]] = go[i];
      if (J) J[group[i]] = gj[i];
      if (evals) evals[group[i]] = ge[i];
    }
    pending.swap(rest);
  }
  return PSR_OK;
}

int psr_refine_grid(const psr_fb *fb, uint64_t n, const psr_timing *start, uint64_t ncand,
                    double resolution_hz, double dm_step, double dm_lo, double dm_hi,
                    uint64_t bins, psr_timing *out, double *rcs) {
  PSR_TRY(refine_length(fb, n));
  if ((!start || !out) && ncand) {
    set_error("refine: null argument");
    return PSR_EINVAL;
  }
  if (!(resolution_hz >= 0.0) || !(dm_step > 0.0) || !(dm_lo >= 0.0) || !(dm_hi >= dm_lo) ||
      bins < 4) {
    set_error("refine_grid: resolution >= 0, dm_step > 0, 0 <= dm_lo <= dm_hi, bins >= 4");
    return PSR_EINVAL;
  }
  for (uint64_t i = 0; i < ncand; ++i) {
    double r = 0.0;
    PSR_TRY(grid_refine_one(fb->o, n, start[i], resolution_hz, dm_step, dm_lo, dm_hi, bins,
                            out[i], r, fb->stream.s));
    if (rcs) rcs[i] = r;
  }
  return PSR_OK;
}

// search::sift (search/src/lib.rs:147-176).
int psr_sift(const psr_candidate *in, uint64_t n, double res, uint64_t limit,
             int reject_dm_zero, psr_candidate *out, uint64_t *n_out) {
  std::vector<psr_candidate> c(in, in + n);
  auto key = [](double x) {
    int64_t i;
    std::memcpy(&i, &x, 8);
    return i ^ (int64_t)((uint64_t)(i >> 63) >> 1);
  };
  std::stable_sort(c.begin(), c.end(), [&](const psr_candidate &a, const psr_candidate &b) {
    return key(a.score) > key(b.score);
  });
  std::vector<psr_candidate> kept;
  std::vector<double> rejected;
  for (const psr_candidate &x : c) {
    auto related = [&](double f) {
      for (int h = 1; h <= 16; ++h)
        if (std::fabs(x.frequency_hz - f * h) <= res || std::fabs(f - x.frequency_hz * h) <= res)
          return true;
      return false;
    };
    bool skip = std::any_of(kept.begin(), kept.end(),
                            [&](const psr_candidate &k) { return related(k.frequency_hz); }) ||
                std::any_of(rejected.begin(), rejected.end(), related);
    if (skip) continue;
    if (reject_dm_zero && x.dm <= 0.0) {
      rejected.push_back(x.frequency_hz);
      continue;
    }
    kept.push_back(x);
    if (kept.size() >= limit) break;
  }
  *n_out = kept.size();
  if (out) std::copy(kept.begin(), kept.end(), out);
  return PSR_OK;
}

int psr_profile_at(const float *series, uint64_t n, double tsamp, double period, uint64_t bins,
                   uint64_t sample_offset, psr_profile_stats *stats, float *values,
                   uint64_t *counts) {
  if (!series || !stats || bins < 4 || !std::isfinite(period) || period <= 0.0 ||
      !std::isfinite(tsamp) || tsamp <= 0.0 || n == 0) {
    set_error("profile_at: bins >= 4, finite positive period/tsamp required");
    return PSR_EINVAL;
  }
  Stream s;
  DevBuf x;
  PSR_TRY(x.ensure(n * 4));
  PSR_CUDA(cudaMemcpyAsync(x.p, series, n * 4, cudaMemcpyHostToDevice, s.s));
  return fold_profiles(x.as<float>(), n, tsamp, &period, 1, bins, sample_offset, stats, values,
                       counts, s.s);
}

int psr_refine(const float *series, uint64_t n, double tsamp, double frequency, double span_hz,
               uint64_t steps, uint64_t bins, psr_profile_stats *stats, float *values,
               uint64_t *counts) {
  if (!series || !stats || steps == 0 || !(frequency > span_hz) || !(span_hz >= 0.0) ||
      bins < 4 || n == 0) {
    set_error("refine: steps > 0 and frequency > span_hz >= 0 required");
    return PSR_EINVAL;
  }
  std::vector<double> periods(steps + 1);
  for (uint64_t i = 0; i <= steps; ++i) {
    const double f = frequency - span_hz + 2.0 * span_hz * (double)i / (double)steps;
    periods[i] = 1.0 / f;
  }
  Stream s;
  DevBuf x;
  PSR_TRY(x.ensure(n * 4));
  PSR_CUDA(cudaMemcpyAsync(x.p, series, n * 4, cudaMemcpyHostToDevice, s.s));
  std::vector<psr_profile_stats> st(steps + 1);
  std::vector<float> vals((steps + 1) * bins);
  std::vector<uint64_t> cnts((steps + 1) * bins);
  PSR_TRY(fold_profiles(x.as<float>(), n, tsamp, periods.data(), steps + 1, bins, 0, st.data(),
                        vals.data(), cnts.data(), s.s));
  // max_by keeps the last maximum (fold/src/lib.rs:93-95).
  uint64_t best = 0;
  auto key = [](double v) {
    int64_t i;
    std::memcpy(&i, &v, 8);
    return i ^ (int64_t)((uint64_t)(i >> 63) >> 1);
  };
  for (uint64_t i = 1; i <= steps; ++i)
    if (key(st[i].reduced_chi_square) >= key(st[best].reduced_chi_square)) best = i;
  *stats = st[best];
  if (values) std::copy(vals.begin() + best * bins, vals.begin() + (best + 1) * bins, values);
  if (counts) std::copy(cnts.begin() + best * bins, cnts.begin() + (best + 1) * bins, counts);
  return PSR_OK;
}

int psr_measure(const float *x, uint64_t n, uint64_t offset, double tsamp, double period,
                uint64_t start_bin, uint64_t width_bins, uint64_t bins, psr_measurement *out) {
  if (!x || !out || bins == 0 || width_bins == 0 || width_bins > bins || start_bin >= bins ||
      !(period > 0.0) || !(tsamp > 0.0) || n == 0) {
    set_error("measure: a valid window, positive period/tsamp and samples are required");
    return PSR_EINVAL;
  }
  Stream s;
  DevBuf d;
  PSR_TRY(d.ensure(n * 4));
  PSR_CUDA(cudaMemcpyAsync(d.p, x, n * 4, cudaMemcpyHostToDevice, s.s));
  return measure_device(d.as<float>(), n, offset, tsamp, period, start_bin, width_bins, bins,
                        out, s.s);
}

// ------------------------------------------------------------ session
namespace {
// psr_session_create with the engine's outer chunk fixed up front (0: the
// default), so that a batch allocates each session's buffers once.
int session_create(const psr_header *header, uint64_t nsamples, const double *trials,
                   uint64_t ntrials, uint64_t discovery, const psr_search_config *cfg,
                   uint64_t rfi_block_samples, float rfi_threshold, uint64_t chunk,
                   psr_session **out) {
  if (!header || !trials || !valid_config(cfg) || !out || nsamples < 2 || header->nchans <= 0) {
    set_error("session: invalid arguments");
    return PSR_EINVAL;
  }
  std::unique_ptr<psr_session> s(new psr_session());
  DeviceObs &o = s->o;
  o.h = *header;
  o.ns = nsamples;
  o.nch = (uint64_t)header->nchans;
  o.kind = kind_for_bits(header->nbits);
  o.payload_bytes = (nsamples * o.nch * (uint64_t)header->nbits + 7) / 8;
  PSR_TRY(o.payload.ensure(o.payload_bytes + 16));
  PSR_TRY(o.alloc(s->stream.s));
  s->rfi_block = rfi_block_samples;
  s->rfi_threshold = rfi_threshold;
  s->trials.assign(trials, trials + ntrials);
  s->discovery = discovery;
  s->spec = to_spec(cfg, header->tsamp);
  s->eng.chunk = chunk;
  PSR_TRY(s->eng.prepare(o, trials, ntrials, discovery, s->spec, s->stream.s));
  PSR_TRY(s->errbuf.ensure(8));
  PSR_CUDA(cudaStreamSynchronize(s->stream.s));
  *out = s.release();
  return PSR_OK;
}
}  // namespace

int psr_session_create(const psr_header *header, uint64_t nsamples, const double *trials,
                       uint64_t ntrials, uint64_t discovery, const psr_search_config *cfg,
                       uint64_t rfi_block_samples, float rfi_threshold, psr_session **out) {
  return session_create(header, nsamples, trials, ntrials, discovery, cfg, rfi_block_samples,
                        rfi_threshold, 0, out);
}

int psr_session_load(psr_session *s, const uint8_t *payload, uint64_t nbytes) {
  if (!s || !payload || nbytes < s->o.payload_bytes) {
    set_error("session_load: payload smaller than the session's observation");
    return PSR_EINVAL;
  }
  PSR_CUDA(cudaMemcpyAsync(s->o.payload.p, payload, s->o.payload_bytes, cudaMemcpyHostToDevice,
                           s->stream.s));
  return PSR_OK;
}

int psr_session_run(psr_session *s) {
  if (!s) {
    set_error("session_run: null handle");
    return PSR_EINVAL;
  }
  cudaStream_t st = s->stream.s;
  PSR_CUDA(cudaMemsetAsync(s->errbuf.p, 0xff, 8, st));
  PSR_TRY(s->mark(0, 0));
  PSR_TRY(launch_unpack(s->o, s->errbuf.as<unsigned long long>(), st));
  PSR_TRY(s->mark(0, 1));
  if (s->rfi_block) {
    PSR_TRY(s->mark(1, 0));
    PSR_TRY(rfi_enqueue(s->o, s->rfi_block, s->rfi_threshold, s->rfi, st));
    PSR_TRY(s->mark(1, 1));
  }
  PSR_TRY(s->eng.enqueue(s->o, st));
  s->have_run = true;
  return PSR_OK;
}

int psr_session_sync(psr_session *s) {
  if (!s || !s->have_run) {
    set_error("session_sync: nothing has been run");
    return PSR_EINVAL;
  }
  cudaStream_t st = s->stream.s;
  PSR_TRY(s->h_err.ensure(8));
  PSR_CUDA(cudaMemcpyAsync(s->h_err.p, s->errbuf.p, 8, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  const unsigned long long e = *s->h_err.as<unsigned long long>();
  if (e != ~0ull) {
    set_error("invalid or unsupported filterbank: nonfinite sample at " +
              std::to_string(e / s->o.nch) + "/" + std::to_string(e % s->o.nch));
    return PSR_EFORMAT;
  }
  PSR_TRY(s->harvest());
  return s->eng.finish(s->o, st);
}

int psr_session_set_profiling(psr_session *s, int enable) {
  if (!s) {
    set_error("session_set_profiling: null handle");
    return PSR_EINVAL;
  }
  if (enable < 0 || enable > 2) {
    set_error("session_set_profiling: 0, 1 or 2");
    return PSR_EINVAL;
  }
  s->eng.profile = enable;
  return PSR_OK;
}

int psr_session_stage_times(psr_session *s, double *ms, uint64_t *launches, int reset) {
  if (!s) {
    set_error("session_stage_times: null handle");
    return PSR_EINVAL;
  }
  const double v[5] = {s->pre_ms[0], s->pre_ms[1], s->eng.stage_ms[0], s->eng.stage_ms[1],
                       s->eng.stage_ms[2]};
  const uint64_t l[5] = {s->pre_launches[0], s->pre_launches[1], s->eng.stage_launches[0],
                         s->eng.stage_launches[1], s->eng.stage_launches[2]};
  for (int i = 0; i < 5; ++i) {
    if (ms) ms[i] = v[i];
    if (launches) launches[i] = l[i];
  }
  if (reset) {
    s->pre_ms[0] = s->pre_ms[1] = 0.0;
    s->pre_launches[0] = s->pre_launches[1] = 0;
    for (int i = 0; i < 3; ++i) {
      s->eng.stage_ms[i] = 0.0;
      s->eng.stage_launches[i] = 0;
    }
  }
  return PSR_OK;
}

int psr_session_candidates(psr_session *s, uint64_t *counts, psr_candidate *out, uint64_t cap,
                           uint64_t *n_total) {
  if (!s || !n_total) {
    set_error("session_candidates: null argument");
    return PSR_EINVAL;
  }
  return s->eng.collect(s->stream.s, counts, out, cap, n_total);
}

int psr_session_mask(psr_session *s, uint64_t *channels, uint64_t *nchannels_bad,
                     uint64_t *blocks, uint64_t blocks_cap, uint64_t *nblocks_bad,
                     double *masked_fraction) {
  if (!s || !nchannels_bad || !nblocks_bad || !masked_fraction) {
    set_error("session_mask: null argument");
    return PSR_EINVAL;
  }
  if (!s->rfi_block) {
    *nchannels_bad = 0;
    *nblocks_bad = 0;
    *masked_fraction = 0.0;
    return PSR_OK;
  }
  RfiResult res;
  PSR_TRY(rfi_collect(s->o, s->rfi_block, s->rfi, s->stream.s, res));
  *nchannels_bad = res.channels.size();
  if (channels) std::copy(res.channels.begin(), res.channels.end(), channels);
  *nblocks_bad = res.blocks.size();
  if (blocks)
    for (uint64_t i = 0; i < res.blocks.size() && i < blocks_cap; ++i) blocks[i] = res.blocks[i];
  *masked_fraction = res.masked_fraction;
  return PSR_OK;
}

void *psr_session_payload_device(psr_session *s) { return s ? s->o.payload.p : nullptr; }
void *psr_session_stream(psr_session *s) { return s ? (void *)s->stream.s : nullptr; }
int psr_session_analyze(psr_session *s, uint64_t limit, uint64_t bins, const psr_rules *rules,
                        psr_outcome **out) {
  if (!s || !out) {
    set_error("session_analyze: null argument");
    return PSR_EINVAL;
  }
  if (!s->have_run) {
    set_error("session_analyze: nothing has been run");
    return PSR_EINVAL;
  }
  PSR_TRY(psr_session_sync(s));
  uint64_t total = 0;
  PSR_TRY(s->eng.collect(s->stream.s, nullptr, nullptr, 0, &total));
  std::vector<psr_candidate> all(total);
  PSR_TRY(s->eng.collect(s->stream.s, nullptr, all.data(), all.size(), &total));
  psr_rules r;
  psr_rules_default(&r);
  std::unique_ptr<psr_outcome> o(new psr_outcome());
  PSR_TRY(analyze_obs(s->o, s->trials.data(), s->trials.size(), all.data(), all.size(), limit,
                      bins, rules ? *rules : r, o->o, s->stream.s));
  *out = o.release();
  return PSR_OK;
}

void psr_session_free(psr_session *s) { delete s; }

// ------------------------------------------------------------------ batch
// Many observations of uneven shape searched by one CUDA graph: each
// observation is a session (its own stream and buffers); the first run after
// any change of the work captures every session's whole pipeline (unpack,
// RFI, all trial chunks) into one graph whose branches run concurrently;
// later runs launch that graph.
struct psr_batch {
  std::vector<std::unique_ptr<psr_session>> obs;
  Stream main;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<cudaEvent_t> events;
  bool warm = false;
  std::vector<uint64_t> chunk, inner;  // chosen by psr_batch_tune (0: defaults)
  ~psr_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (cudaEvent_t e : events) cudaEventDestroy(e);
  }
  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    warm = false;
  }
};

namespace {
// Trials per dedispersion launch so that the batch's dedispersed series and
// spectra stay within `budget` bytes of HBM (at least 16 per observation).
uint64_t chunk_for_budget(const psr_batch_obs *obs, uint64_t n, double budget) {
  double per_trial = 0.0;
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t len = obs[i].discovery;
    uint64_t p = 1;
    while (p < len) p <<= 1;
    // series, two halves of power spectra, FFT work buffer (complex, p points)
    per_trial += 4.0 * (double)series_ld(len) + 8.0 * (double)(p + 64) + 8.0 * (double)p;
  }
  const double c = per_trial > 0.0 ? budget / per_trial : 256.0;
  return (uint64_t)std::max(16.0, std::min(256.0, std::floor(c)));
}

int reprepare(psr_session *s, uint64_t chunk, uint64_t inner, int subbands = -2) {
  s->eng.chunk = chunk;
  s->eng.inner = inner;
  if (subbands > -2) s->eng.subbands = subbands;
  PSR_TRY(s->eng.prepare(s->o, s->trials.data(), s->trials.size(), s->discovery, s->spec,
                         s->stream.s));
  PSR_CUDA(cudaStreamSynchronize(s->stream.s));
  return PSR_OK;
}
}  // namespace

int psr_batch_create(const psr_batch_obs *obs, uint64_t n, uint64_t hbm_budget_bytes,
                     psr_batch **out) {
  if (!obs || n == 0 || !out) {
    set_error("batch: invalid arguments");
    return PSR_EINVAL;
  }
  std::unique_ptr<psr_batch> b(new psr_batch());
  const double budget = hbm_budget_bytes ? (double)hbm_budget_bytes : 64.0 * (1ull << 30);
  const uint64_t chunk = chunk_for_budget(obs, n, budget);
  for (uint64_t i = 0; i < n; ++i) {
    const psr_batch_obs &q = obs[i];
    psr_session *s = nullptr;
    PSR_TRY(session_create(&q.header, q.nsamples, q.trials, q.ntrials, q.discovery, &q.config,
                           q.rfi_block_samples, q.rfi_threshold, chunk, &s));
    b->obs.emplace_back(s);
    b->chunk.push_back(s->eng.chunk);
    b->inner.push_back(s->eng.inner);
  }
  *out = b.release();
  return PSR_OK;
}

int psr_batch_load(psr_batch *b, uint64_t i, const uint8_t *payload, uint64_t nbytes) {
  if (!b || i >= b->obs.size()) {
    set_error("batch: observation index out of range");
    return PSR_EINVAL;
  }
  return psr_session_load(b->obs[i].get(), payload, nbytes);
}

int psr_batch_load_fb(psr_batch *b, uint64_t i, const psr_fb *fb) {
  if (!b || i >= b->obs.size() || !fb) {
    set_error("batch: observation index out of range");
    return PSR_EINVAL;
  }
  psr_session *s = b->obs[i].get();
  if (fb->o.nch != s->o.nch || fb->o.ns != s->o.ns || s->o.h.nbits != 8) {
    set_error("batch: the filterbank's shape differs from the observation's");
    return PSR_EINVAL;
  }
  PSR_CUDA(cudaStreamSynchronize(fb->stream.s));
  PSR_TRY(pack_payload_u8(fb->o, s->o.payload.as<uint8_t>(), s->stream.s));
  PSR_CUDA(cudaStreamSynchronize(s->stream.s));
  return PSR_OK;
}

int psr_batch_set_chunking(psr_batch *b, uint64_t i, uint64_t chunk, uint64_t inner) {
  if (!b || i >= b->obs.size() || chunk == 0) {
    set_error("batch: observation index out of range or empty DM block");
    return PSR_EINVAL;
  }
  b->drop_graph();
  psr_session *s = b->obs[i].get();
  PSR_TRY(reprepare(s, chunk, inner));
  b->chunk[i] = s->eng.chunk;
  b->inner[i] = s->eng.inner;
  return PSR_OK;
}

// Autotuner.  Observations fall into shape classes (channels, bit depth, FFT
// size, trial count to the nearest power of two); the first observation of a
// class is searched whole at each candidate tiling, on its loaded data, and
// the fastest is applied to the whole class.  Candidates: the budgeted DM
// block and half of it (outer chunk), whole-block or 64-trial FFT launches
// (inner chunk), and for 8-bit samples channel-by-channel or 8-channel
// subband dedispersion.
int psr_batch_tune(psr_batch *b, uint64_t *chunk_out, uint64_t *inner_out, int *subbands_out) {
  if (!b) {
    set_error("batch: null handle");
    return PSR_EINVAL;
  }
  b->drop_graph();
  struct Pick {
    uint64_t chunk, inner;
    int subbands;
  };
  std::map<std::tuple<uint64_t, int64_t, uint64_t, int>, Pick> classes;
  cudaEvent_t e0, e1;
  PSR_CUDA(cudaEventCreate(&e0));
  PSR_CUDA(cudaEventCreate(&e1));
  int rc = PSR_OK;
  for (size_t i = 0; i < b->obs.size() && rc == PSR_OK; ++i) {
    psr_session *s = b->obs[i].get();
    int lt = 0;
    while ((1ull << lt) < s->trials.size()) ++lt;
    const auto key = std::make_tuple(s->o.nch, s->o.h.nbits, s->eng.fft.M, lt);
    auto it = classes.find(key);
    if (it == classes.end()) {
      const uint64_t c0 = b->chunk[i];
      std::vector<Pick> cand;
      for (uint64_t c : {c0, std::max<uint64_t>(16, c0 / 2)})
        for (uint64_t inner : {(uint64_t)0, (uint64_t)64})
          for (int g : {0, 8})
            if (g == 0 || s->o.h.nbits == 8) cand.push_back(Pick{c, inner, g});
      double best = 1e300;
      Pick pick = cand[0];
      for (const Pick &c : cand) {
        if ((rc = reprepare(s, c.chunk, c.inner, c.subbands)) != PSR_OK) break;
        if ((rc = psr_session_run(s)) != PSR_OK || (rc = psr_session_sync(s)) != PSR_OK) break;
        if (cudaEventRecord(e0, s->stream.s) != cudaSuccess ||
            (rc = psr_session_run(s)) != PSR_OK ||
            cudaEventRecord(e1, s->stream.s) != cudaSuccess ||
            (rc = psr_session_sync(s)) != PSR_OK) {
          if (rc == PSR_OK) rc = PSR_ECUDA;
          break;
        }
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
          rc = PSR_ECUDA;
          break;
        }
        if (ms < best) {
          best = ms;
          pick = Pick{s->eng.chunk, s->eng.inner, c.subbands};
        }
      }
      it = classes.emplace(key, pick).first;
    }
    if (rc != PSR_OK) break;
    const Pick &p = it->second;
    rc = reprepare(s, p.chunk, p.inner, p.subbands);
    b->chunk[i] = p.chunk;
    b->inner[i] = p.inner;
    if (chunk_out) chunk_out[i] = p.chunk;
    if (inner_out) inner_out[i] = p.inner;
    if (subbands_out) subbands_out[i] = p.subbands;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

int psr_batch_run(psr_batch *b) {
  if (!b) {
    set_error("batch: null handle");
    return PSR_EINVAL;
  }
  if (!b->warm) {
    // One direct run settles every buffer and kernel attribute, so that the
    // capture below records stream work only.
    for (auto &s : b->obs) PSR_TRY(psr_session_run(s.get()));
    for (auto &s : b->obs) PSR_TRY(psr_session_sync(s.get()));
    b->warm = true;
  }
  if (!b->exec) {
    cudaStream_t m = b->main.s;
    for (cudaEvent_t e : b->events) cudaEventDestroy(e);
    b->events.assign(b->obs.size() + 1, nullptr);
    for (auto &e : b->events) PSR_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    PSR_CUDA(cudaStreamBeginCapture(m, cudaStreamCaptureModeRelaxed));
    int rc = PSR_OK;
    rc = cudaEventRecord(b->events[0], m) == cudaSuccess ? PSR_OK : PSR_ECUDA;
    for (size_t i = 0; i < b->obs.size() && rc == PSR_OK; ++i) {
      psr_session *s = b->obs[i].get();
      if (cudaStreamWaitEvent(s->stream.s, b->events[0], 0) != cudaSuccess) rc = PSR_ECUDA;
      if (rc == PSR_OK) rc = psr_session_run(s);
      if (rc == PSR_OK && cudaEventRecord(b->events[i + 1], s->stream.s) != cudaSuccess)
        rc = PSR_ECUDA;
      if (rc == PSR_OK && cudaStreamWaitEvent(m, b->events[i + 1], 0) != cudaSuccess)
        rc = PSR_ECUDA;
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(m, &g);
    if (rc != PSR_OK || ec != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      if (rc == PSR_OK) set_error(std::string("batch: graph capture failed: ") +
                                  cudaGetErrorString(ec));
      return rc == PSR_OK ? PSR_ECUDA : rc;
    }
    b->graph = g;
    PSR_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
  }
  PSR_CUDA(cudaGraphLaunch(b->exec, b->main.s));
  for (auto &s : b->obs) s->have_run = true;
  return PSR_OK;
}

int psr_batch_sync(psr_batch *b) {
  if (!b) {
    set_error("batch: null handle");
    return PSR_EINVAL;
  }
  PSR_CUDA(cudaStreamSynchronize(b->main.s));
  bool regrown = false;
  for (auto &s : b->obs) {
    // A raw-candidate overflow makes finish() regrow that session's buffers
    // and redo the chunk; the captured graph would then hold stale pointers,
    // so it is captured again on the next run.
    const void *raw = s->eng.sw.raw.p, *gq = s->eng.sw.gq.p;
    PSR_TRY(psr_session_sync(s.get()));
    regrown = regrown || s->eng.sw.raw.p != raw || s->eng.sw.gq.p != gq;
  }
  if (regrown) b->drop_graph();
  return PSR_OK;
}

int psr_batch_candidates(psr_batch *b, uint64_t i, uint64_t *counts, psr_candidate *out,
                         uint64_t cap, uint64_t *n_total) {
  if (!b || i >= b->obs.size()) {
    set_error("batch: observation index out of range");
    return PSR_EINVAL;
  }
  return psr_session_candidates(b->obs[i].get(), counts, out, cap, n_total);
}

void *psr_batch_stream(psr_batch *b) { return b ? (void *)b->main.s : nullptr; }

void psr_batch_free(psr_batch *b) { delete b; }

}  // extern "C"
