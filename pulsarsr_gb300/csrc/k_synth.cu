// Seeded synthetic filterbanks generated on the device (the psr synth
// command and the large test shapes).  The reference's generator
// (synth/src/lib.rs:37-88) draws its noise from ChaCha8 + Ziggurat (rand
// 0.8.8), which is not reproduced; this one keeps its signal model:
//   x[c][t] = mean + sigma * gain_c * (n(c, t) + sum_p pulse_p(c, t)),
//   pulse_p = A_p exp(-0.5 (d / (duty_p / 2.355))^2), d = distance of the phase
//   (t*tsamp - delay_c) / P - pdot (t*tsamp - delay_c)^2 / (2 P^2) - phase0
//   from the nearest integer, delay_c = K DM (f_c^-2 - f_max^-2) (fractional),
// quantised with round-to-nearest and clamped for integer bit depths.
// n(c, t) is N(0, 1) from a counter-based hash of (seed, c, t) (SplitMix64
// finaliser; Box-Muller), so any sample can be generated independently and
// the same seed always gives the same data.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "psr_internal.h"

namespace psr {
namespace {

constexpr int SY_NT = 256;
constexpr int SY_PER = 32;  // samples per thread, strided by SY_NT
constexpr int SY_MAXP = 64;

struct SynthPulsarDev {
  double nu, nudot, phase0;  // 1/P, -pdot/P^2, phase offset (cycles)
  float amp, inv_width;      // A, 2.355 / duty
};

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

template <class T>
__global__ void __launch_bounds__(SY_NT)
    k_synth(T *__restrict__ out, uint64_t ld, uint64_t ns, uint64_t seed, double tsamp,
            float mean, float sigma, const float *__restrict__ gain,
            const SynthPulsarDev *__restrict__ ps, const double *__restrict__ delay, int np,
            uint64_t nch, float hi) {
  const uint64_t c = blockIdx.y;
  const uint64_t t0 = (uint64_t)blockIdx.x * SY_NT * SY_PER + threadIdx.x;
  const float gsig = sigma * gain[c];
  float acc[SY_PER];
#pragma unroll
  for (int j = 0; j < SY_PER; ++j) {
    const uint64_t t = t0 + (uint64_t)j * SY_NT;
    const uint64_t h = mix64(seed ^ mix64(c * 0x100000001B3ull + t));
    const float u1 = ((float)(uint32_t)(h >> 40) + 1.0f) * (1.0f / 16777216.0f);  // (0, 1]
    const float u2 = (float)(uint32_t)(h & 0xffffffu) * (1.0f / 16777216.0f);     // [0, 1)
    acc[j] = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
  }
  for (int p = 0; p < np; ++p) {
    const SynthPulsarDev q = ps[p];
    // Phase at this thread's first sample in f64; steps of SY_NT samples in f32.
    const double td = (double)t0 * tsamp - delay[(uint64_t)p * nch + c];
    const double ph = q.nu * td + 0.5 * q.nudot * td * td - q.phase0;
    const float base = (float)(ph - floor(ph));
    const float step = (float)((q.nu + q.nudot * td) * tsamp * (double)SY_NT);
#pragma unroll
    for (int j = 0; j < SY_PER; ++j) {
      float f = base + step * (float)j;
      f -= floorf(f);
      const float d = fminf(f, 1.0f - f) * q.inv_width;
      acc[j] += q.amp * __expf(-0.5f * d * d);
    }
  }
#pragma unroll
  for (int j = 0; j < SY_PER; ++j) {
    const uint64_t t = t0 + (uint64_t)j * SY_NT;
    if (t >= ns) continue;
    float v = mean + gsig * acc[j];
    if (hi > 0.0f) v = fminf(fmaxf(rintf(v), 0.0f), hi);
    out[c * ld + t] = (T)v;
  }
}

inline uint64_t host_mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

int synth_obs(const psr_synth_config &cfg, DeviceObs &o, cudaStream_t st) {
  if (cfg.nchans < 1 || cfg.nsamples < 2 || !(cfg.tsamp > 0.0) || !std::isfinite(cfg.tsamp) ||
      !(cfg.nbits == 8 || cfg.nbits == 16 || cfg.nbits == 32 || cfg.nbits == 1 ||
        cfg.nbits == 2 || cfg.nbits == 4) ||
      cfg.npulsars > (uint64_t)SY_MAXP || (cfg.npulsars && !cfg.pulsars) ||
      !(cfg.noise_sigma >= 0.0) || !(cfg.gain_spread >= 0.0 && cfg.gain_spread < 1.0)) {
    set_error("invalid synthetic configuration");
    return PSR_EINVAL;
  }
  const uint64_t nch = (uint64_t)cfg.nchans;
  double fmax = 0.0;
  for (uint64_t c = 0; c < nch; ++c) {
    const double f = cfg.fch1 + (double)c * cfg.foff;
    if (!(f > 0.0) || !std::isfinite(f)) {
      set_error("invalid synthetic configuration");
      return PSR_EINVAL;
    }
    fmax = std::fmax(fmax, f);
  }
  std::vector<SynthPulsarDev> ps(cfg.npulsars);
  std::vector<double> delay(cfg.npulsars * nch);
  for (uint64_t p = 0; p < cfg.npulsars; ++p) {
    const psr_synth_pulsar &q = cfg.pulsars[p];
    if (!(q.period_s > 0.0) || !(q.duty > 0.0 && q.duty < 0.5) || !(q.amplitude >= 0.0) ||
        !(q.dm >= 0.0) || !std::isfinite(q.pdot)) {
      set_error("invalid synthetic configuration");
      return PSR_EINVAL;
    }
    ps[p] = SynthPulsarDev{1.0 / q.period_s, -q.pdot / (q.period_s * q.period_s), q.phase,
                           (float)q.amplitude, (float)(2.355 / q.duty)};
    for (uint64_t c = 0; c < nch; ++c) {
      const double f = cfg.fch1 + (double)c * cfg.foff;
      delay[p * nch + c] = 4148.808 * q.dm * (1.0 / (f * f) - 1.0 / (fmax * fmax));
    }
  }
  std::vector<float> gain(nch);
  for (uint64_t c = 0; c < nch; ++c) {
    const uint64_t h = host_mix64(cfg.seed ^ host_mix64(0xC0FFEEull + c));
    const double u = (double)(h >> 11) * (1.0 / 9007199254740992.0);
    gain[c] = (float)(1.0 + cfg.gain_spread * (2.0 * u - 1.0));
  }
  o.h = psr_header{cfg.nchans, cfg.nbits, cfg.tsamp, cfg.fch1, cfg.foff, 0};
  o.ns = cfg.nsamples;
  o.nch = nch;
  o.kind = kind_for_bits(cfg.nbits);
  PSR_TRY(o.alloc(st));
  DevBuf dgain, dps, ddelay;
  PSR_TRY(dgain.ensure(nch * 4));
  PSR_TRY(dps.ensure(ps.size() * sizeof(SynthPulsarDev) + 16));
  PSR_TRY(ddelay.ensure(delay.size() * 8 + 16));
  PSR_CUDA(cudaMemcpyAsync(dgain.p, gain.data(), nch * 4, cudaMemcpyHostToDevice, st));
  if (!ps.empty()) {
    PSR_CUDA(cudaMemcpyAsync(dps.p, ps.data(), ps.size() * sizeof(SynthPulsarDev),
                             cudaMemcpyHostToDevice, st));
    PSR_CUDA(cudaMemcpyAsync(ddelay.p, delay.data(), delay.size() * 8, cudaMemcpyHostToDevice,
                             st));
  }
  const uint64_t seed = host_mix64(cfg.seed);
  const float hi = cfg.nbits <= 16 ? (float)((1u << cfg.nbits) - 1) : 0.0f;
  dim3 grid((unsigned)((o.ns + SY_NT * SY_PER - 1) / (SY_NT * SY_PER)), (unsigned)nch);
  const float mean = (float)cfg.noise_mean, sigma = (float)cfg.noise_sigma;
  switch (o.kind) {
    case SAMPLE_U8:
      k_synth<uint8_t><<<grid, SY_NT, 0, st>>>(
          o.samples.as<uint8_t>(), o.ld, o.ns, seed, cfg.tsamp, mean, sigma, dgain.as<float>(),
          dps.as<SynthPulsarDev>(), ddelay.as<double>(), (int)ps.size(), nch, hi);
      break;
    case SAMPLE_U16:
      k_synth<uint16_t><<<grid, SY_NT, 0, st>>>(
          o.samples.as<uint16_t>(), o.ld, o.ns, seed, cfg.tsamp, mean, sigma, dgain.as<float>(),
          dps.as<SynthPulsarDev>(), ddelay.as<double>(), (int)ps.size(), nch, hi);
      break;
    default:
      k_synth<float><<<grid, SY_NT, 0, st>>>(
          o.samples.as<float>(), o.ld, o.ns, seed, cfg.tsamp, mean, sigma, dgain.as<float>(),
          dps.as<SynthPulsarDev>(), ddelay.as<double>(), (int)ps.size(), nch, 0.0f);
  }
  PSR_CUDA(cudaGetLastError());
  PSR_CUDA(cudaStreamSynchronize(st));
  return PSR_OK;
}

namespace {
// Interference added in place: channel c of `band` (1 = narrowband) gets
// nb_amp * (0.5 + 0.5 sin(2 pi nb_hz t tsamp + phi_c)) on every sample; every
// channel gets burst_amp inside each burst window [start_k, start_k + width).
// Values are rounded and clamped again for integer bit depths.
template <class T>
__global__ void __launch_bounds__(SY_NT)
    k_inject_rfi(T *__restrict__ out, uint64_t ld, uint64_t ns, double tsamp,
                 const uint8_t *__restrict__ band, const float *__restrict__ phi, float nb_amp,
                 double nb_hz, const uint64_t *__restrict__ starts, int nbursts, uint64_t width,
                 float burst_amp, float hi) {
  const uint64_t c = blockIdx.y;
  const bool nb = band[c] != 0;
  for (uint64_t t = (uint64_t)blockIdx.x * SY_NT + threadIdx.x; t < ns;
       t += (uint64_t)gridDim.x * SY_NT) {
    float add = 0.0f;
    if (nb) {
      const double x = nb_hz * tsamp * (double)t;
      add += nb_amp * (0.5f + 0.5f * sinpif(2.0f * (float)(x - floor(x)) + phi[c]));
    }
    for (int k = 0; k < nbursts; ++k)
      if (t >= starts[k] && t - starts[k] < width) add += burst_amp;
    if (add == 0.0f) continue;
    float v = (float)out[c * ld + t] + add;
    if (hi > 0.0f) v = fminf(fmaxf(rintf(v), 0.0f), hi);
    out[c * ld + t] = (T)v;
  }
}

// payload[t * nch + c] = samples[c * ld + t] for 8-bit samples: 32 x 32
// tiles through shared memory (coalesced reads along t, writes along c).
__global__ void k_pack_u8(const uint8_t *__restrict__ samples, uint64_t ld, uint64_t ns,
                          uint64_t nch, uint8_t *__restrict__ payload) {
  __shared__ uint8_t tile[32][33];
  const uint64_t t0 = (uint64_t)blockIdx.x * 32, c0 = (uint64_t)blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const uint64_t c = c0 + r, t = t0 + threadIdx.x;
    tile[r][threadIdx.x] = (c < nch && t < ns) ? samples[c * ld + t] : 0;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const uint64_t t = t0 + r, c = c0 + threadIdx.x;
    if (t < ns && c < nch) payload[t * nch + c] = tile[threadIdx.x][r];
  }
}
}  // namespace

int inject_rfi(DeviceObs &o, const psr_synth_rfi &r, cudaStream_t st) {
  if (r.nb_channels > o.nch || r.nbursts > 1024 || !(r.nb_amplitude >= 0.0) ||
      !(r.burst_amplitude >= 0.0) || !std::isfinite(r.nb_hz) ||
      (r.nbursts && (r.burst_samples == 0 || r.burst_samples > o.ns))) {
    set_error("invalid interference configuration");
    return PSR_EINVAL;
  }
  // Seeded choices: narrowband channels (distinct), their tone phases and
  // the burst start samples.
  std::vector<uint8_t> band(o.nch, 0);
  std::vector<float> phi(o.nch, 0.0f);
  uint64_t picked = 0, i = 0;
  while (picked < r.nb_channels) {
    const uint64_t c = host_mix64(r.seed ^ host_mix64(0xBA5Eull + i++)) % o.nch;
    if (!band[c]) {
      band[c] = 1;
      ++picked;
    }
  }
  for (uint64_t c = 0; c < o.nch; ++c)
    phi[c] = (float)((host_mix64(r.seed ^ host_mix64(0xF00Dull + c)) >> 40) *
                     (2.0 / 16777216.0));
  std::vector<uint64_t> starts(r.nbursts + 1, 0);
  for (uint64_t k = 0; k < r.nbursts; ++k)
    starts[k] = host_mix64(r.seed ^ host_mix64(0xB0B0ull + k)) % (o.ns - r.burst_samples + 1);
  DevBuf dband, dphi, dstarts;
  PSR_TRY(dband.ensure(o.nch));
  PSR_TRY(dphi.ensure(o.nch * 4));
  PSR_TRY(dstarts.ensure(starts.size() * 8));
  PSR_CUDA(cudaMemcpyAsync(dband.p, band.data(), o.nch, cudaMemcpyHostToDevice, st));
  PSR_CUDA(cudaMemcpyAsync(dphi.p, phi.data(), o.nch * 4, cudaMemcpyHostToDevice, st));
  PSR_CUDA(cudaMemcpyAsync(dstarts.p, starts.data(), starts.size() * 8, cudaMemcpyHostToDevice,
                           st));
  const float hi = o.kind == SAMPLE_U8 ? (float)((1u << (o.h.nbits < 8 ? o.h.nbits : 8)) - 1)
                   : o.kind == SAMPLE_U16 ? 65535.0f : 0.0f;
  dim3 grid((unsigned)std::min<uint64_t>((o.ns + SY_NT - 1) / SY_NT, 64), (unsigned)o.nch);
  const float nba = (float)r.nb_amplitude, ba = (float)r.burst_amplitude;
  switch (o.kind) {
    case SAMPLE_U8:
      k_inject_rfi<uint8_t><<<grid, SY_NT, 0, st>>>(
          o.samples.as<uint8_t>(), o.ld, o.ns, o.h.tsamp, dband.as<uint8_t>(), dphi.as<float>(),
          nba, r.nb_hz, dstarts.as<uint64_t>(), (int)r.nbursts, r.burst_samples, ba, hi);
      break;
    case SAMPLE_U16:
      k_inject_rfi<uint16_t><<<grid, SY_NT, 0, st>>>(
          o.samples.as<uint16_t>(), o.ld, o.ns, o.h.tsamp, dband.as<uint8_t>(), dphi.as<float>(),
          nba, r.nb_hz, dstarts.as<uint64_t>(), (int)r.nbursts, r.burst_samples, ba, hi);
      break;
    default:
      k_inject_rfi<float><<<grid, SY_NT, 0, st>>>(
          o.samples.as<float>(), o.ld, o.ns, o.h.tsamp, dband.as<uint8_t>(), dphi.as<float>(),
          nba, r.nb_hz, dstarts.as<uint64_t>(), (int)r.nbursts, r.burst_samples, ba, 0.0f);
  }
  PSR_CUDA(cudaGetLastError());
  PSR_CUDA(cudaStreamSynchronize(st));
  return PSR_OK;
}

int pack_payload_u8(const DeviceObs &src, uint8_t *d_payload, cudaStream_t st) {
  if (src.kind != SAMPLE_U8 || src.h.nbits != 8) {
    set_error("batch: device observations must hold 8-bit samples");
    return PSR_EINVAL;
  }
  dim3 grid((unsigned)((src.ns + 31) / 32), (unsigned)((src.nch + 31) / 32));
  k_pack_u8<<<grid, dim3(32, 8), 0, st>>>(src.samples.as<uint8_t>(), src.ld, src.ns, src.nch,
                                           d_payload);
  PSR_CUDA(cudaGetLastError());
  return PSR_OK;
}

}  // namespace psr
