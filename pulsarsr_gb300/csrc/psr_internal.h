// Internal declarations shared by the libpsr translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

#include <string>
#include <vector>

#include "../../include/psr.h"

namespace psr {

// ------------------------------------------------------------ errors
void set_error(const std::string &msg);
const std::string &last_error();

struct Status {
  int code = PSR_OK;
  bool ok() const { return code == PSR_OK; }
};

#define PSR_CUDA(call)                                                     \
  do {                                                                     \
    cudaError_t e_ = (call);                                               \
    if (e_ != cudaSuccess) {                                               \
      ::psr::set_error(std::string("CUDA error in ") + #call + ": " +      \
                       cudaGetErrorString(e_));                            \
      return PSR_ECUDA;                                                    \
    }                                                                      \
  } while (0)

#define PSR_TRY(expr)                 \
  do {                                \
    int rc_ = (expr);                 \
    if (rc_ != PSR_OK) return rc_;    \
  } while (0)

// Binary exponent of the finest quantum of a finite f32 value: x is an
// integer multiple of 2^quantum_exponent(x); zero constrains nothing.  A
// set of f32 values with finest quantum 2^q has every partial f64 sum exact,
// in any order, while the sum of their magnitudes stays below 2^(53+q).
constexpr int kNoQuantum = 1 << 20;
#ifdef __CUDACC__
__device__ __forceinline__ int quantum_exponent(float x) {
  const uint32_t b = __float_as_uint(x) & 0x7fffffffu;
  if (b == 0) return kNoQuantum;
  const int e = (int)(b >> 23);
  uint32_t m = b & 0x7fffffu;
  if (e) m |= 0x800000u;
  return (e ? e : 1) - 150 + (__ffs((int)m) - 1);
}
#endif
// True when sums of magnitude at most `mag` over values whose finest quantum
// is 2^q are exact in f64 whatever the order (mag itself rounded: a margin).
__host__ __device__ inline bool f64_sums_exact(double mag, int q) {
  return q >= kNoQuantum || mag * (1.0 + 0x1p-20) < ldexp(1.0, 53 + q);
}

// Owning device allocation (sized once, reused).
// Page-locked host memory, grown on demand and kept across calls (device
// copies into it run at full link speed, with no staging and no page faults).
struct HostBuf {
  void *p = nullptr;
  size_t bytes = 0;
  HostBuf() = default;
  HostBuf(const HostBuf &) = delete;
  HostBuf &operator=(const HostBuf &) = delete;
  ~HostBuf() { release(); }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
  }
  int ensure(size_t n) {
    if (n <= bytes && p) return PSR_OK;
    release();
    if (n == 0) n = 16;
    cudaError_t e = cudaHostAlloc(&p, n, cudaHostAllocDefault);
    if (e != cudaSuccess) {
      p = nullptr;
      set_error(std::string("CUDA error in cudaHostAlloc(") + std::to_string(n) +
                " bytes): " + cudaGetErrorString(e));
      return PSR_ECUDA;
    }
    bytes = n;
    return PSR_OK;
  }
  template <class T>
  T *as() const {
    return static_cast<T *>(p);
  }
};

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  int ensure(size_t n) {
    if (n <= bytes && p) return PSR_OK;
    release();
    if (n == 0) n = 16;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
      p = nullptr;
      set_error(std::string("CUDA error in cudaMalloc(") + std::to_string(n) +
                " bytes): " + cudaGetErrorString(e));
      return PSR_ECUDA;
    }
    bytes = n;
    return PSR_OK;
  }
  template <class T>
  T *as() const {
    return static_cast<T *>(p);
  }
};

// Sample storage type of the device filterbank.
enum SampleKind { SAMPLE_U8 = 0, SAMPLE_U16 = 1, SAMPLE_F32 = 2 };

inline int sample_bytes(SampleKind k) { return k == SAMPLE_U8 ? 1 : (k == SAMPLE_U16 ? 2 : 4); }
inline SampleKind kind_for_bits(int64_t nbits) {
  return nbits <= 8 ? SAMPLE_U8 : (nbits == 16 ? SAMPLE_U16 : SAMPLE_F32);
}

// Channel-major samples on the device: row c starts at c*ld elements.  ld is
// a multiple of 64 elements and rows carry >= 64 elements of zero padding so
// that 16-byte aligned tile copies never leave the allocation.
struct DeviceObs {
  psr_header h{};
  uint64_t ns = 0;
  uint64_t nch = 0;
  SampleKind kind = SAMPLE_U8;
  uint64_t ld = 0;
  DevBuf samples;
  DevBuf payload;   // packed bytes as read (time-major)
  uint64_t payload_bytes = 0;
  int alloc(cudaStream_t st);  // samples for (nch, ns, kind), zeroed on st
  // Maximum sample value (integer kinds) used for exactness decisions.
  double max_value() const {
    if (kind == SAMPLE_U8) return (double)((1u << (h.nbits < 8 ? h.nbits : 8)) - 1);
    if (kind == SAMPLE_U16) return 65535.0;
    return 0.0;
  }
};

// Seeded synthetic observation generated on the device (k_synth.cu).
int synth_obs(const psr_synth_config &cfg, DeviceObs &o, cudaStream_t st);
// Seeded interference added in place (narrowband channels, broadband bursts).
int inject_rfi(DeviceObs &o, const psr_synth_rfi &r, cudaStream_t st);
// Time-major 8-bit payload (as read from a file) of a device observation.
int pack_payload_u8(const DeviceObs &src, uint8_t *d_payload, cudaStream_t st);

// Host-side restatements that stay on the host (FP64 tables, small sorts).
bool host_delays(const double *f, size_t n, double tsamp, double dm,
                 std::vector<uint64_t> &out);
int parse_header(const uint8_t *b, uint64_t len, psr_header &h);

// ---------------------------------------------------------- kernels
// Unpack the packed time-major payload into channel-major samples.
// err_index receives min(t*nch+ch) of a non-finite f32 sample (or ~0).
int launch_unpack(const DeviceObs &o, unsigned long long *d_err_index,
                  cudaStream_t st);

// RFI mask (rfi::mask) on the device samples.  Scratch is owned by RfiWork.
struct RfiWork {
  DevBuf means, vars, med, bsum, bmeans, chbad, blkbad, scratch, flags, hist, mhist;
  uint64_t blocks_n = 0;
};
struct RfiResult {
  std::vector<uint64_t> channels, blocks;
  double masked_fraction = 0.0;
};
int rfi_enqueue(DeviceObs &o, uint64_t block_samples, float threshold,
                RfiWork &w, cudaStream_t st);
int rfi_collect(const DeviceObs &o, uint64_t block_samples, RfiWork &w,
                cudaStream_t st, RfiResult &res);
// The per-channel means and variances rfi::mask computes, to host arrays.
int rfi_channel_stats(const DeviceObs &o, float *means, float *variances, cudaStream_t st);

// Exact upper median of n device floats (radix select), result to d_out.
int launch_median_f32(const float *d_vals, uint64_t n, float *d_out,
                      unsigned int *d_hist_scratch, cudaStream_t st);


// ---------------------------------------------------------- spectra
struct FftPlan {
  uint64_t len = 0;   // series length
  uint64_t N = 0;     // real FFT size
  uint64_t M = 0;     // complex size N/2
  int m = 0;          // log2 M
  uint64_t M1 = 0, M2 = 0;
  DevBuf Q;           // quarter twiddle table, N/4 + 1 float2
  DevBuf tw1;         // pass-1 twiddles W_M^(n2*k1) laid out [k1][n2]
  int init(uint64_t series_len, cudaStream_t st);
  uint64_t bins() const { return M + 1; }
  uint64_t pass2_ctas() const;
};

struct SpecConfig {
  double tsamp = 0;
  double min_hz = 1, max_hz = 0, threshold = 6;
  uint64_t max_candidates = 32;
  std::vector<double> birdies;  // pairs
  int levels = 5;               // harmonic sums h = 1 .. 2^(levels-1)
};
struct SpecWork {
  DevBuf scale, raw, raw_count, birdies, overflow, gq, gn;
  uint64_t qcap = 0;          // gate queue capacity per trial
  bool queue_full = false;    // size the gate queues for every bin
  uint64_t outer_trials = 0;  // trials of the chunk being processed
  uint64_t raw_cap = 0;  // raw (pre-dedupe) candidates per trial
  uint64_t lds = 0;      // row stride of scale[]
};
int spectrum_prepare(const FftPlan &p, const SpecConfig &c, uint64_t outer, uint64_t inner,
                     SpecWork &w, cudaStream_t st);
int spectrum_reset(SpecWork &w, uint64_t outer_trials, cudaStream_t st);
int spectrum_gate(const FftPlan &p, const SpecConfig &c, const float *d_power, uint64_t ldp,
                  const double *d_psum, uint32_t npsum, uint64_t ntrials, uint64_t slot0,
                  SpecWork &w, cudaStream_t st);
int spectrum_items(const FftPlan &p, const SpecConfig &c, const float *d_power, uint64_t ldp,
                   uint64_t ntrials, SpecWork &w, cudaStream_t st);
int spectrum_select(const FftPlan &p, const SpecConfig &c, const double *d_trial_dm,
                    uint64_t ntrials, SpecWork &w, psr_candidate *d_kept, unsigned *d_kept_count,
                    cudaStream_t st);

// Row stride (floats) of a dedispersed series buffer of length n.
uint64_t series_ld(uint64_t n);
// Delay table [ntrials][nch] (u32) for the trial DMs, the widest delay spread
// of a channel within 8 consecutive trials, and the largest delay.
int make_delay_table(const DeviceObs &o, const double *trials, uint64_t ntrials,
                     std::vector<uint32_t> &tab, uint64_t &max_spread, uint64_t &max_delay);
// out[trial][t] (row stride ldo); sums[trial] = f64 series sum, means[trial] =
// (f32)(sum / n), the value search::periodicity subtracts.  The staged
// (packed integer) kernel's waits give up after spin_limit polls (0 = the
// default limit) and set *d_err; arm_only = 1 arms its barriers without
// issuing the copies, so every wait runs out (a test of that path).
// Subband-reuse plan of the staged dedispersion kernel for one DM plan
// split into outer chunks (k_dedisperse.cu): per block of 8 consecutive
// trials of a chunk and subband of G adjacent channels, the distinct
// intra-subband delay patterns.  G = 0: no plan.
struct SubbandPlan {
  int G = 0;
  uint64_t nsub = 0;
  DevBuf entries;
  std::vector<uint64_t> block0;  // first block of each outer chunk
  uint64_t reused = 0, direct = 0;  // (block, subband) pairs by mode
};
// The subband width searches use when not told otherwise: the process-wide
// setting of psr_set_dedisp_subbands, else the per-sample-kind default.
int dedisp_subbands_default(const DeviceObs &o);
int build_subband_plan(const std::vector<uint32_t> &tab, uint64_t nch,
                       const std::vector<uint64_t> &cstart, int G, SubbandPlan &plan,
                       cudaStream_t st);
// With want_means = false (series only folded, not searched) the sums and
// means are left unset.  With a subband plan (8-bit-storage samples), chunk
// chunk_index of the plan runs the subband-reuse kernel.
int launch_dedisperse_ex(const DeviceObs &o, const uint32_t *d_delays, uint64_t ntrials,
                         uint64_t n, float *d_out, uint64_t ldo, double *d_part, double *d_sums,
                         float *d_means, uint64_t max_spread, unsigned *d_err, cudaStream_t st,
                         long long spin_limit = 0, int arm_only = 0, bool want_means = true,
                         const SubbandPlan *sb = nullptr, uint64_t chunk_index = 0);
uint64_t dedisperse_part_count(const DeviceObs &o, uint64_t n);
// The f64 sum of a device series and the f32 mean search::periodicity
// subtracts (search/src/lib.rs:36), bit-identical to the reference's
// sequential sum: added in parallel where that is exact, else in order.  One
// CTA; d_sum may be null.
int launch_series_mean(const float *d_x, uint64_t n, double *d_sum, float *d_mean,
                       cudaStream_t st);
int launch_raw_power_ex(const FftPlan &p, const float *d_series, uint64_t lds,
                        const float *d_means, uint64_t ntrials, float2 *d_work, float *d_power,
                        uint64_t ldp, double *d_psum, cudaStream_t st);
// The same kernels with caller-owned twiddle tables (FftPlan's Q and tw1
// layouts for real FFT size N = 2 * next_pow2(len)); N <= 2^21.
int launch_raw_power_tables(uint64_t len, uint64_t N, const float2 *d_Q, const float2 *d_tw1,
                            const float *d_series, uint64_t lds, const float *d_means,
                            uint64_t ntrials, float2 *d_work, float *d_power, uint64_t ldp,
                            double *d_psum, cudaStream_t st);

// ------------------------------------------------------------- fold
// Host statistics of a folded profile (fold/src/lib.rs:39-79).
void profile_stats(const double *sums, const unsigned long long *cnts, uint64_t bins,
                   double smean, double svar, double period, psr_profile_stats *st,
                   float *values, uint64_t *counts);
// confirmation::measure on a device series.
int measure_device(const float *d_x, uint64_t n, uint64_t offset, double tsamp, double period,
                   uint64_t start_bin, uint64_t width_bins, uint64_t bins, psr_measurement *out,
                   cudaStream_t st);
int fold_profiles(const float *d_series, uint64_t n, double tsamp,
                  const double *periods, uint64_t nper, uint64_t bins,
                  uint64_t sample_offset, psr_profile_stats *stats,
                  float *values, uint64_t *counts, cudaStream_t st);
// nper (series, period) pairs, series p at d_series + p * xstride.
int fold_profiles_ex(const float *d_series, uint64_t xstride, uint64_t n, double tsamp,
                     const double *periods, uint64_t nper, uint64_t bins,
                     uint64_t sample_offset, psr_profile_stats *stats, float *values,
                     uint64_t *counts, cudaStream_t st);
// fold::profile of every channel row of o over samples [0, n): values[c*bins+b].
int fold_channels(const DeviceObs &o, uint64_t n, double tsamp, double period, uint64_t bins,
                  std::vector<float> &values, cudaStream_t st);
// Combined shifted channel profiles per trial (confirmation.rs:397-413):
// comb[trial*bins + b]; d_delays is the [ntrials][nch] u32 delay table.
int dm_response(const std::vector<float> &chp, const std::vector<double> &chmean,
                const uint32_t *d_delays, uint64_t ntrials, uint64_t nch, uint64_t bins,
                double tsamp, double period, std::vector<double> &comb, cudaStream_t st);

}  // namespace psr
