// psr_raw_power_noalloc: the raw power spectrum of search::periodicity
// (search/src/lib.rs:35-44) computed by the same FFT kernels as psr_raw_power,
// with every byte of device scratch taken from one file-scope static device
// array instead of cudaMalloc.
//
// Who needs it: callers that must not allocate device memory while they run —
// a process whose device memory is handed out up front to another pool (a
// framework's caching allocator, an MPS client under a memory limit), and
// real-time callers that cannot take the device-wide synchronisation that
// cudaFree performs while other streams are busy.  psr_raw_power allocates and
// frees its series, work and twiddle buffers on every call; this entry point
// reserves them once, when the module is loaded on a device.
//
// The array lives in this translation unit only, so only processes that call
// this entry point load it (CUDA loads modules lazily).
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "psr_internal.h"

namespace psr {
namespace {

constexpr uint64_t align256(uint64_t b) { return (b + 255) / 256 * 256; }

// Largest series: 2^20 samples, so N = 2^21 real points and M = 2^20 complex.
constexpr uint64_t NA_MAX_LEN = PSR_RAW_POWER_NOALLOC_MAX_LEN;
constexpr uint64_t NA_MAX_M = NA_MAX_LEN;
constexpr uint64_t NA_MAX_N = 2 * NA_MAX_M;
// Pass-2 partial sums: at most 129 CTAs for M up to 2^20.
constexpr uint64_t NA_MAX_PSUM = 512;

// Region offsets (bytes) inside the array; each region is 256-byte aligned.
constexpr uint64_t NA_SER = 0;                                          // series, f32
constexpr uint64_t NA_MEAN = NA_SER + align256(NA_MAX_LEN * 4 + 256);   // (f32)mean
constexpr uint64_t NA_WORK = NA_MEAN + 256;                             // four-step work, float2
constexpr uint64_t NA_POW = NA_WORK + align256(NA_MAX_M * 8 + 16);      // power, f32
constexpr uint64_t NA_PSUM = NA_POW + align256((NA_MAX_M + 1 + 64) * 4);  // partial sums, f64
constexpr uint64_t NA_Q = NA_PSUM + align256(NA_MAX_PSUM * 8);          // quarter table, float2
constexpr uint64_t NA_TW1 = NA_Q + align256((NA_MAX_N / 4 + 1) * 8);    // pass-1 twiddles
constexpr uint64_t NA_BYTES = NA_TW1 + align256(NA_MAX_M * 8);

static_assert(NA_BYTES < (32ull << 20), "scratch stays below 32 MiB");

// The scratch.  No region has to start at zero: the FFT kernels read the
// series only below len, and every other region is written before it is read
// within one call.
static __device__ __align__(256) unsigned char g_raw_power_scratch[NA_BYTES];

constexpr int NA_MAX_DEVICES = 64;
struct DeviceScratch {
  unsigned char *base = nullptr;  // address of g_raw_power_scratch on the device
  uint64_t table_N = 0;           // FFT size whose twiddles the Q/TW1 regions hold
};
DeviceScratch g_devices[NA_MAX_DEVICES];
std::mutex g_setup_mu;

// Once per device, with that device current: look up the array's address.
int scratch_for_current_device(DeviceScratch **out) {
  int dev = 0;
  PSR_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= NA_MAX_DEVICES) {
    set_error("raw_power_noalloc: device ordinal " + std::to_string(dev) + " above " +
              std::to_string(NA_MAX_DEVICES - 1));
    return PSR_EINVAL;
  }
  std::lock_guard<std::mutex> lock(g_setup_mu);
  DeviceScratch &d = g_devices[dev];
  if (!d.base) {
    void *p = nullptr;
    PSR_CUDA(cudaGetSymbolAddress(&p, g_raw_power_scratch));
    d.base = static_cast<unsigned char *>(p);
  }
  *out = &d;
  return PSR_OK;
}

// Quarter-wave twiddle Q[r], r in [0, N/4]: (cos, sin)(2*pi*r/N) rounded to f32
// for r <= N/8 and the swapped mirror above, the table FftPlan::init builds.
float2 quarter_entry(uint64_t N, uint64_t r) {
  const uint64_t n8 = N / 8, n4 = N / 4;
  if (r > n8) {
    const float2 v = quarter_entry(N, n4 - r);
    return make_float2(v.y, v.x);
  }
  const double a = 6.283185307179586 * (double)r / (double)N;
  return make_float2((float)std::cos(a), (float)std::sin(a));
}

// W_N^x from the quarter table and the quadrant of x, as the kernels look it up.
float2 twiddle_entry(uint64_t N, uint64_t x) {
  const uint64_t n4 = N / 4;
  const float2 v = quarter_entry(N, x % n4);
  switch ((x / n4) & 3) {
    case 0: return make_float2(v.x, -v.y);
    case 1: return make_float2(-v.y, -v.x);
    case 2: return make_float2(-v.x, v.y);
    default: return make_float2(v.y, v.x);
  }
}

// Writes the twiddle tables for FFT size N into the Q and TW1 regions through
// a stack buffer (pageable copies return once the driver has staged the
// buffer, so it can be refilled at once).
int write_tables(unsigned char *base, uint64_t N, cudaStream_t st) {
  constexpr uint64_t CH = 2048;
  float2 buf[CH];
  const uint64_t nq = N / 4 + 1;
  float2 *dq = reinterpret_cast<float2 *>(base + NA_Q);
  for (uint64_t i = 0; i < nq; i += CH) {
    const uint64_t c = nq - i < CH ? nq - i : CH;
    for (uint64_t j = 0; j < c; ++j) buf[j] = quarter_entry(N, i + j);
    PSR_CUDA(cudaMemcpyAsync(dq + i, buf, c * sizeof(float2), cudaMemcpyHostToDevice, st));
  }
  const uint64_t M = N / 2;
  int m = 0;
  while ((1ull << m) < M) ++m;
  if (m > 12) {
    // tw1[k1 * M2 + n2] = W_N^(2 * n2 * k1).
    const uint64_t M2 = 1ull << (m / 2);
    float2 *dt = reinterpret_cast<float2 *>(base + NA_TW1);
    for (uint64_t i = 0; i < M; i += CH) {
      const uint64_t c = M - i < CH ? M - i : CH;
      for (uint64_t j = 0; j < c; ++j) {
        const uint64_t e = i + j, k1 = e / M2, n2 = e % M2;
        buf[j] = twiddle_entry(N, 2 * n2 * k1);
      }
      PSR_CUDA(cudaMemcpyAsync(dt + i, buf, c * sizeof(float2), cudaMemcpyHostToDevice, st));
    }
  }
  return PSR_OK;
}

// Pass-2 CTAs per trial for complex size M (FftPlan::pass2_ctas).
uint64_t pass2_ctas_for(uint64_t M) {
  int m = 0;
  while ((1ull << m) < M) ++m;
  if (m <= 12) return 1;
  const uint64_t M1 = 1ull << ((m + 1) / 2), M2 = 1ull << (m / 2);
  const uint64_t C = M2 >= 8192 ? 1 : (8192 / M2 < 16 ? 8192 / M2 : 16);
  const uint64_t H = C / 2;
  return 1 + (M1 / 2 - 1 + H - 1) / H;
}

}  // namespace
}  // namespace psr

using namespace psr;

extern "C" int psr_raw_power_noalloc(const float *series, uint64_t len, float *out,
                                     void *stream) {
  if (!series || !out || len < 2) {
    set_error("periodicity: series of at least two samples required");
    return PSR_EINVAL;
  }
  if (len > NA_MAX_LEN) {
    set_error("raw_power_noalloc: series of " + std::to_string(len) +
              " samples exceeds the fixed scratch maximum of " + std::to_string(NA_MAX_LEN) +
              " samples (use psr_raw_power)");
    return PSR_ECAPACITY;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  DeviceScratch *d = nullptr;
  PSR_TRY(scratch_for_current_device(&d));
  uint64_t M = 1;
  while (M < len) M <<= 1;
  const uint64_t N = 2 * M;
  if (pass2_ctas_for(M) > NA_MAX_PSUM) {
    set_error("raw_power_noalloc: partial-sum region too small");
    return PSR_ECAPACITY;
  }
  unsigned char *base = d->base;
  if (d->table_N != N) {
    d->table_N = 0;
    PSR_TRY(write_tables(base, N, st));
    d->table_N = N;
  }
  float *d_ser = reinterpret_cast<float *>(base + NA_SER);
  float *d_mean = reinterpret_cast<float *>(base + NA_MEAN);
  float *d_pow = reinterpret_cast<float *>(base + NA_POW);
  PSR_CUDA(cudaMemcpyAsync(d_ser, series, len * 4, cudaMemcpyHostToDevice, st));
  // The mean as psr_raw_power takes it (one CTA, no scratch of its own).
  PSR_TRY(launch_series_mean(d_ser, len, nullptr, d_mean, st));
  const uint64_t lds = series_ld(len), ldp = ((M + 1 + 63) / 64) * 64;
  PSR_TRY(launch_raw_power_tables(len, N, reinterpret_cast<const float2 *>(base + NA_Q),
                                  reinterpret_cast<const float2 *>(base + NA_TW1), d_ser, lds,
                                  d_mean, 1, reinterpret_cast<float2 *>(base + NA_WORK), d_pow,
                                  ldp, reinterpret_cast<double *>(base + NA_PSUM), st));
  PSR_CUDA(cudaMemcpyAsync(out, d_pow, (M + 1) * 4, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  return PSR_OK;
}
