// K8 folding (fold::profile_at, fold/src/lib.rs:16-80) and K9 grid refinement
// (fold::refine, fold/src/lib.rs:81-97) for many trial periods in one launch.
//
// bin(t) = min(floor(fract(((t + offset) * tsamp) / period) * bins), bins-1)
// in f64 exactly as the reference.  Bin sums are f64; the per-CTA partial
// sums are combined in a fixed order.  For integer-valued series (sums of
// integer samples) every partial sum is an exact integer, so the result is
// independent of the order and equals the reference's sequential sum.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "psr_internal.h"

namespace psr {
namespace {

constexpr int FOLD_NT = 256;
constexpr int FOLD_MAXBINS = 1024;

__global__ void __launch_bounds__(FOLD_NT)
    k_fold(const float *__restrict__ x, uint64_t xstride, uint64_t n, double tsamp,
           const double *__restrict__ periods, uint64_t bins, uint64_t offset,
           uint64_t per_cta, double *__restrict__ psums, unsigned long long *__restrict__ pcounts) {
  extern __shared__ unsigned char sm_raw[];
  double *s = reinterpret_cast<double *>(sm_raw);
  unsigned *c = reinterpret_cast<unsigned *>(s + bins);
  const uint64_t per = blockIdx.y;
  const double period = periods[per];
  x += per * xstride;
  for (uint64_t b = threadIdx.x; b < bins; b += blockDim.x) {
    s[b] = 0.0;
    c[b] = 0;
  }
  __syncthreads();
  const uint64_t t0 = (uint64_t)blockIdx.x * per_cta;
  const uint64_t t1 = min(t0 + per_cta, n);
  const double dbins = (double)bins;
  for (uint64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
    const double q = __ddiv_rn(__dmul_rn((double)(t + offset), tsamp), period);
    const double ph = __dsub_rn(q, trunc(q));
    uint64_t b = (uint64_t)__dmul_rn(ph, dbins);
    if (b > bins - 1) b = bins - 1;
    atomicAdd(&s[b], (double)x[t]);
    atomicAdd(&c[b], 1u);
  }
  __syncthreads();
  const uint64_t slot = (per * gridDim.x + blockIdx.x) * bins;
  for (uint64_t b = threadIdx.x; b < bins; b += blockDim.x) {
    psums[slot + b] = s[b];
    pcounts[slot + b] = c[b];
  }
}

__global__ void k_fold_reduce(const double *__restrict__ psums,
                              const unsigned long long *__restrict__ pcounts, uint64_t nparts,
                              uint64_t bins, uint64_t nper, double *__restrict__ sums,
                              unsigned long long *__restrict__ counts) {
  const uint64_t id = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= nper * bins) return;
  const uint64_t per = id / bins, b = id % bins;
  double s = 0.0;
  unsigned long long cnt = 0;
  for (uint64_t p = 0; p < nparts; ++p) {
    s += psums[(per * nparts + p) * bins + b];
    cnt += pcounts[(per * nparts + p) * bins + b];
  }
  sums[id] = s;
  counts[id] = cnt;
}

// Series mean and variance in f64 (fold/src/lib.rs:63-68), for series at
// x + blockIdx.y * xstride: pass 1 sums each CTA's slice (partials), pass 2
// (k_series_var) sums (x - mean)^2 with the mean taken from all partials.
constexpr int MOM_NT = 256, MOM_PER = 8192;
__global__ void __launch_bounds__(MOM_NT)
    k_series_sum(const float *__restrict__ x, uint64_t xstride, uint64_t n,
                 double *__restrict__ parts) {
  __shared__ double red[MOM_NT / 32];
  x += blockIdx.y * xstride;
  const uint64_t t0 = (uint64_t)blockIdx.x * MOM_PER, t1 = min(t0 + MOM_PER, n);
  double acc = 0.0;
  for (uint64_t t = t0 + threadIdx.x; t < t1; t += MOM_NT) acc += (double)x[t];
  for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < MOM_NT / 32; ++w) s += red[w];
    parts[blockIdx.y * gridDim.x + blockIdx.x] = s;
  }
}

__global__ void __launch_bounds__(MOM_NT)
    k_series_var(const float *__restrict__ x, uint64_t xstride, uint64_t n,
                 const double *__restrict__ sparts, uint32_t nparts,
                 double *__restrict__ vparts) {
  __shared__ double red[MOM_NT / 32];
  __shared__ double mean_s;
  x += blockIdx.y * xstride;
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (uint32_t i = 0; i < nparts; ++i) s += sparts[blockIdx.y * nparts + i];
    mean_s = s / (double)n;
  }
  __syncthreads();
  const double m = mean_s;
  const uint64_t t0 = (uint64_t)blockIdx.x * MOM_PER, t1 = min(t0 + MOM_PER, n);
  double acc = 0.0;
  for (uint64_t t = t0 + threadIdx.x; t < t1; t += MOM_NT) {
    const double d = __dsub_rn((double)x[t], m);
    acc = __dadd_rn(acc, __dmul_rn(d, d));
  }
  for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < MOM_NT / 32; ++w) s += red[w];
    vparts[blockIdx.y * gridDim.x + blockIdx.x] = s;
  }
}

// confirmation::measure (search/src/confirmation.rs:107-141): on/off sums.
// Each warp covers 32 consecutive samples per step, so the on/off decision
// of every sample also lands in `bits` (one word per 32 samples) for the
// sequential pass.  part[block][8] = n0, s0, q0, n1, s1, q1, sum |v|, and the
// finest quantum exponent among the values (as a double).
constexpr int MEAS_NT = 256;
__global__ void __launch_bounds__(MEAS_NT)
    k_measure(const float *__restrict__ x, uint64_t n, uint64_t offset, double tsamp,
              double period, uint64_t start_bin, uint64_t width_bins, uint64_t bins,
              double *__restrict__ part, uint32_t *__restrict__ bits) {
  __shared__ double red[7][MEAS_NT / 32];
  __shared__ int redq[MEAS_NT / 32];
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};  // n0, s0, q0, n1, s1, q1, sum |v|
  int qm = kNoQuantum;
  const double dbins = (double)bins;
  const int lane = threadIdx.x & 31;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n;
       base += stride) {  // warp-uniform: base is a multiple of 32
    const uint64_t i = base + lane;
    int k = 0;
    if (i < n) {
      const double q = __ddiv_rn(__dmul_rn((double)(i + offset), tsamp), period);
      uint64_t b = (uint64_t)__dmul_rn(__dsub_rn(q, trunc(q)), dbins);
      if (b > bins - 1) b = bins - 1;
      k = ((b + bins - start_bin) % bins) < width_bins ? 1 : 0;
      const float xf = x[i];
      const double v = (double)xf;
      acc[3 * k] += 1.0;
      acc[3 * k + 1] = __dadd_rn(acc[3 * k + 1], v);
      acc[3 * k + 2] = __dadd_rn(acc[3 * k + 2], __dmul_rn(v, v));
      acc[6] = __dadd_rn(acc[6], fabs(v));
      qm = min(qm, quantum_exponent(xf));
    }
    const unsigned w = __ballot_sync(0xffffffffu, k);
    if (lane == 0) bits[base >> 5] = w;
  }
#pragma unroll
  for (int j = 0; j < 7; ++j) {
    double a = acc[j];
    for (int o = 16; o; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) red[j][threadIdx.x >> 5] = a;
  }
  for (int o = 16; o; o >>= 1) qm = min(qm, __shfl_down_sync(0xffffffffu, qm, o));
  if (lane == 0) redq[threadIdx.x >> 5] = qm;
  __syncthreads();
  if (threadIdx.x < 7) {
    double a = 0.0;
    for (int w = 0; w < MEAS_NT / 32; ++w) a += red[threadIdx.x][w];
    part[blockIdx.x * 8 + threadIdx.x] = a;
  } else if (threadIdx.x == 7) {
    int q = kNoQuantum;
    for (int w = 0; w < MEAS_NT / 32; ++w) q = min(q, redq[w]);
    part[blockIdx.x * 8 + 7] = (double)q;
  }
}

// The reference's own order for the on/off sums: one thread adds every
// sample in turn (each class from 0.0), as measure() does.  Used when the
// values make a reassociated f64 sum inexact (non-integer series).
__global__ void k_measure_seq(const float *__restrict__ x, uint64_t n,
                              const uint32_t *__restrict__ bits, double *__restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s0 = 0.0, q0 = 0.0, s1 = 0.0, q1 = 0.0;
  for (uint64_t i = 0; i < n; ++i) {
    const double v = (double)x[i];
    const double v2 = __dmul_rn(v, v);
    if ((bits[i >> 5] >> (i & 31)) & 1u) {
      s1 = __dadd_rn(s1, v);
      q1 = __dadd_rn(q1, v2);
    } else {
      s0 = __dadd_rn(s0, v);
      q0 = __dadd_rn(q0, v2);
    }
  }
  out[0] = s0;
  out[1] = q0;
  out[2] = s1;
  out[3] = q1;
}

int32_t key32(float x) {
  int32_t i;
  std::memcpy(&i, &x, 4);
  return i ^ (int32_t)((uint32_t)(i >> 31) >> 1);
}
bool tless(float a, float b) { return key32(a) < key32(b); }

float upper_median(std::vector<float> v) {
  if (v.empty()) return 0.0f;
  size_t i = v.size() / 2;
  std::nth_element(v.begin(), v.begin() + i, v.end(), tless);
  return v[i];
}

}  // namespace

// Profile statistics from bin sums/counts (fold/src/lib.rs:39-79), host.
void profile_stats(const double *sums, const unsigned long long *cnts, uint64_t bins,
                   double smean, double svar, double period, psr_profile_stats *st,
                   float *values, uint64_t *counts) {
  std::vector<float> vals(bins);
  for (uint64_t b = 0; b < bins; ++b)
    vals[b] = cnts[b] > 0 ? (float)(sums[b] / (double)cnts[b]) : 0.0f;
  const float center = upper_median(vals);
  std::vector<float> off;
  for (uint64_t b = 0; b < bins; ++b)
    if (cnts[b] > 0) off.push_back(vals[b]);
  std::sort(off.begin(), off.end(), tless);
  off.resize(std::max<size_t>(off.size() * 3 / 4, 1));
  double mean = -0.0;
  for (float v : off) mean += (double)v;
  mean /= (double)off.size();
  double var = -0.0;
  for (float v : off) {
    const double d = (double)v - mean;
    var += d * d;
  }
  const double sigma = std::sqrt(var / (double)off.size());
  float peak = -INFINITY;
  for (float v : vals) peak = std::fmax(peak, v);
  st->period_s = period;
  st->snr = sigma > 1e-12 ? ((double)peak - (double)center) / sigma : 0.0;
  uint64_t populated = 0;
  for (uint64_t b = 0; b < bins; ++b) populated += cnts[b] > 0;
  if (svar > 1e-12 && populated > 1) {
    double s = -0.0;
    for (uint64_t b = 0; b < bins; ++b) {
      const double d = (double)vals[b] - smean;
      s += (double)cnts[b] * (d * d) / svar;
    }
    st->reduced_chi_square = s / (double)(populated - 1);
  } else {
    st->reduced_chi_square = 0.0;
  }
  if (values) std::copy(vals.begin(), vals.end(), values);
  if (counts)
    for (uint64_t b = 0; b < bins; ++b) counts[b] = cnts[b];
}

int fold_profiles(const float *d_x, uint64_t n, double tsamp, const double *periods,
                  uint64_t nper, uint64_t bins, uint64_t offset, psr_profile_stats *stats,
                  float *values, uint64_t *counts, cudaStream_t st) {
  return fold_profiles_ex(d_x, 0, n, tsamp, periods, nper, bins, offset, stats, values, counts,
                          st);
}

// Fold nper (series, period) pairs: series p starts at d_x + p * xstride
// (xstride 0: one series at every period); stats/values/counts are arrays of
// nper entries (values/counts nper*bins).
int fold_profiles_ex(const float *d_x, uint64_t xstride, uint64_t n, double tsamp,
                     const double *periods, uint64_t nper, uint64_t bins, uint64_t offset,
                     psr_profile_stats *stats, float *values, uint64_t *counts,
                     cudaStream_t st) {
  if (bins < 4 || bins > FOLD_MAXBINS || n == 0) {
    set_error("profile_at: 4 <= bins <= 1024 and a non-empty series are required");
    return PSR_EINVAL;
  }
  const uint64_t per_cta = 8192;
  const uint64_t nparts = (n + per_cta - 1) / per_cta;
  DevBuf dper, psums, pcounts, sums, cnts;
  PSR_TRY(dper.ensure(nper * 8));
  PSR_TRY(psums.ensure(nper * nparts * bins * 8));
  PSR_TRY(pcounts.ensure(nper * nparts * bins * 8));
  PSR_TRY(sums.ensure(nper * bins * 8));
  PSR_TRY(cnts.ensure(nper * bins * 8));
  const uint64_t nser = xstride ? nper : 1;
  PSR_CUDA(cudaMemcpyAsync(dper.p, periods, nper * 8, cudaMemcpyHostToDevice, st));
  const size_t smem = bins * (8 + 4);
  dim3 grid((unsigned)nparts, (unsigned)nper);
  k_fold<<<grid, FOLD_NT, smem, st>>>(d_x, xstride, n, tsamp, dper.as<double>(), bins, offset,
                                      per_cta, psums.as<double>(),
                                      pcounts.as<unsigned long long>());
  PSR_CUDA(cudaGetLastError());
  k_fold_reduce<<<(unsigned)((nper * bins + 255) / 256), 256, 0, st>>>(
      psums.as<double>(), pcounts.as<unsigned long long>(), nparts, bins, nper,
      sums.as<double>(), cnts.as<unsigned long long>());
  const uint32_t mparts = (uint32_t)((n + MOM_PER - 1) / MOM_PER);
  DevBuf sp, vp;
  PSR_TRY(sp.ensure((size_t)nser * mparts * 8));
  PSR_TRY(vp.ensure((size_t)nser * mparts * 8));
  k_series_sum<<<dim3(mparts, (unsigned)nser), MOM_NT, 0, st>>>(d_x, xstride, n,
                                                               sp.as<double>());
  k_series_var<<<dim3(mparts, (unsigned)nser), MOM_NT, 0, st>>>(d_x, xstride, n,
                                                               sp.as<double>(), mparts,
                                                               vp.as<double>());
  PSR_CUDA(cudaGetLastError());
  std::vector<double> hs(nper * bins), hm(2 * nser), hsp((size_t)nser * mparts),
      hvp((size_t)nser * mparts);
  std::vector<unsigned long long> hc(nper * bins);
  PSR_CUDA(cudaMemcpyAsync(hs.data(), sums.p, nper * bins * 8, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaMemcpyAsync(hc.data(), cnts.p, nper * bins * 8, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaMemcpyAsync(hsp.data(), sp.p, hsp.size() * 8, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaMemcpyAsync(hvp.data(), vp.p, hvp.size() * 8, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  for (uint64_t m = 0; m < nser; ++m) {
    double s1 = 0.0, s2 = 0.0;
    for (uint32_t i = 0; i < mparts; ++i) {
      s1 += hsp[m * mparts + i];
      s2 += hvp[m * mparts + i];
    }
    hm[2 * m] = s1;
    hm[2 * m + 1] = s2;
  }
  for (uint64_t p = 0; p < nper; ++p) {
    const uint64_t m = xstride ? p : 0;
    const double smean = hm[2 * m] / (double)n;
    const double svar = hm[2 * m + 1] / (double)n;
    profile_stats(hs.data() + p * bins, hc.data() + p * bins, bins, smean, svar, periods[p],
                  &stats[p], values ? values + p * bins : nullptr,
                  counts ? counts + p * bins : nullptr);
  }
  return PSR_OK;
}

}  // namespace psr

namespace psr {

int measure_device(const float *d_x, uint64_t n, uint64_t offset, double tsamp, double period,
                   uint64_t start_bin, uint64_t width_bins, uint64_t bins, psr_measurement *out,
                   cudaStream_t st) {
  const unsigned nb = (unsigned)std::min<uint64_t>((n + 1023) / 1024, 1024);
  DevBuf part, bits;
  PSR_TRY(part.ensure((size_t)nb * 8 * 8 + 4 * 8));
  PSR_TRY(bits.ensure(((n + 31) / 32 + 1) * 4));
  k_measure<<<nb, MEAS_NT, 0, st>>>(d_x, n, offset, tsamp, period, start_bin, width_bins, bins,
                                    part.as<double>(), bits.as<uint32_t>());
  PSR_CUDA(cudaGetLastError());
  std::vector<double> h((size_t)nb * 8);
  PSR_CUDA(cudaMemcpyAsync(h.data(), part.p, h.size() * 8, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  double a[7] = {0, 0, 0, 0, 0, 0, 0};
  int qmin = kNoQuantum;
  for (unsigned b = 0; b < nb; ++b) {
    for (int j = 0; j < 7; ++j) a[j] += h[(size_t)b * 8 + j];
    qmin = std::min(qmin, (int)h[(size_t)b * 8 + 7]);
  }
  const uint64_t cnt[2] = {(uint64_t)a[0], (uint64_t)a[3]};
  double sum[2] = {a[1], a[4]}, sum2[2] = {a[2], a[5]};
  // Integer-valued series (sums of integer samples) give exact partial sums
  // in any order.  Otherwise the order matters: sums of v are exact while
  // sum |v| < 2^(53+q), sums of v^2 (multiples of 2^2q) while
  // sum v^2 < 2^(53+2q); failing either, add in the reference's order.
  const bool exact = f64_sums_exact(a[6], qmin) &&
                     (qmin >= kNoQuantum || f64_sums_exact(a[2] + a[5], 2 * qmin));
  if (!exact) {
    double *d_seq = part.as<double>() + (size_t)nb * 8;
    k_measure_seq<<<1, 32, 0, st>>>(d_x, n, bits.as<uint32_t>(), d_seq);
    PSR_CUDA(cudaGetLastError());
    double hq[4];
    PSR_CUDA(cudaMemcpyAsync(hq, d_seq, sizeof(hq), cudaMemcpyDeviceToHost, st));
    PSR_CUDA(cudaStreamSynchronize(st));
    sum[0] = hq[0];
    sum2[0] = hq[1];
    sum[1] = hq[2];
    sum2[1] = hq[3];
  }
  out->on_samples = cnt[1];
  out->off_samples = cnt[0];
  if (cnt[0] < 2 || cnt[1] < 2) {
    out->snr = 0.0;
    out->mean_difference = 0.0;
    out->standard_error = 0.0;
    return PSR_OK;
  }
  const double diff = sum[1] / (double)cnt[1] - sum[0] / (double)cnt[0];
  auto var = [&](int k) {
    return std::fmax((sum2[k] - sum[k] * sum[k] / (double)cnt[k]) / (double)(cnt[k] - 1), 0.0);
  };
  const double err = std::sqrt(var(1) / (double)cnt[1] + var(0) / (double)cnt[0]);
  out->snr = err > 1e-10 ? diff / err : 0.0;
  out->mean_difference = diff;
  out->standard_error = err;
  return PSR_OK;
}

}  // namespace psr

// ---------------------------------------------------------------------------
// Per-channel discovery profiles and the DM response of
// confirmation::analyze (search/src/confirmation.rs:391-433).
namespace psr {
namespace {

template <typename T>
__device__ __forceinline__ double sample_as_f64(const T *row, uint64_t t) {
  return (double)(float)row[t];
}

// fold::profile of every channel row over samples [0, n) at one period:
// CTA (part, channel) accumulates its part of the row into shared bins.
template <typename T>
__global__ void __launch_bounds__(FOLD_NT)
    k_fold_rows(const T *__restrict__ samples, uint64_t ld, uint64_t n, double tsamp,
                double period, uint64_t bins, uint64_t per_cta, double *__restrict__ psums,
                unsigned long long *__restrict__ pcounts) {
  extern __shared__ unsigned char sm_raw[];
  double *s = reinterpret_cast<double *>(sm_raw);
  unsigned *c = reinterpret_cast<unsigned *>(s + bins);
  const uint64_t ch = blockIdx.y;
  const T *row = samples + ch * ld;
  for (uint64_t b = threadIdx.x; b < bins; b += blockDim.x) {
    s[b] = 0.0;
    c[b] = 0;
  }
  __syncthreads();
  const uint64_t t0 = (uint64_t)blockIdx.x * per_cta;
  const uint64_t t1 = min(t0 + per_cta, n);
  const double dbins = (double)bins;
  for (uint64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
    const double q = __ddiv_rn(__dmul_rn((double)t, tsamp), period);
    uint64_t b = (uint64_t)__dmul_rn(__dsub_rn(q, trunc(q)), dbins);
    if (b > bins - 1) b = bins - 1;
    atomicAdd(&s[b], sample_as_f64(row, t));
    atomicAdd(&c[b], 1u);
  }
  __syncthreads();
  const uint64_t slot = (ch * gridDim.x + blockIdx.x) * bins;
  for (uint64_t b = threadIdx.x; b < bins; b += blockDim.x) {
    psums[slot + b] = s[b];
    pcounts[slot + b] = c[b];
  }
}

// comb[trial][b] = sum over channels (in channel order) of the linearly
// interpolated, mean-removed channel profile shifted by delay*tsamp/period
// bins; the f64 operations and their order follow confirmation.rs:403-413.
// One CTA per trial; the channel shifts are computed once into shared memory.
__global__ void k_dm_response(const float *__restrict__ chp, const double *__restrict__ chmean,
                              const uint32_t *__restrict__ delays, uint64_t nch, uint64_t bins,
                              double tsamp, double period, double *__restrict__ comb) {
  extern __shared__ double shift[];
  const uint64_t trial = blockIdx.x;
  const double dbins = (double)bins;
  for (uint64_t c = threadIdx.x; c < nch; c += blockDim.x) {
    const double d = (double)delays[trial * nch + c];
    shift[c] = __dmul_rn(__ddiv_rn(__dmul_rn(d, tsamp), period), dbins);
  }
  __syncthreads();
  for (uint64_t b = threadIdx.x; b < bins; b += blockDim.x) {
    double out = 0.0;
    for (uint64_t c = 0; c < nch; ++c) {
      double pos = fmod(__dadd_rn((double)b, shift[c]), dbins);
      if (pos < 0.0) pos = __dadd_rn(pos, dbins);
      const double fl = floor(pos);
      uint64_t index = (uint64_t)fl;
      if (index > bins - 1) index = bins - 1;
      const double fraction = __dsub_rn(pos, (double)index);
      const double m = chmean[c];
      const double a = __dmul_rn(__dsub_rn((double)chp[c * bins + index], m),
                                 __dsub_rn(1.0, fraction));
      const double e = __dmul_rn(__dsub_rn((double)chp[c * bins + (index + 1) % bins], m),
                                 fraction);
      out = __dadd_rn(out, __dadd_rn(a, e));
    }
    comb[trial * bins + b] = out;
  }
}

}  // namespace

int fold_channels(const DeviceObs &o, uint64_t n, double tsamp, double period, uint64_t bins,
                  std::vector<float> &values, cudaStream_t st) {
  if (bins < 4 || bins > FOLD_MAXBINS || n == 0 || n > o.ns) {
    set_error("profile: 4 <= bins <= 1024 and 0 < n <= nsamples are required");
    return PSR_EINVAL;
  }
  const uint64_t per_cta = 8192;
  const uint64_t nparts = (n + per_cta - 1) / per_cta;
  DevBuf psums, pcounts, sums, cnts;
  PSR_TRY(psums.ensure(o.nch * nparts * bins * 8));
  PSR_TRY(pcounts.ensure(o.nch * nparts * bins * 8));
  PSR_TRY(sums.ensure(o.nch * bins * 8));
  PSR_TRY(cnts.ensure(o.nch * bins * 8));
  const size_t smem = bins * (8 + 4);
  dim3 grid((unsigned)nparts, (unsigned)o.nch);
  switch (o.kind) {
    case SAMPLE_U8:
      k_fold_rows<unsigned char><<<grid, FOLD_NT, smem, st>>>(
          o.samples.as<unsigned char>(), o.ld, n, tsamp, period, bins, per_cta,
          psums.as<double>(), pcounts.as<unsigned long long>());
      break;
    case SAMPLE_U16:
      k_fold_rows<uint16_t><<<grid, FOLD_NT, smem, st>>>(
          o.samples.as<uint16_t>(), o.ld, n, tsamp, period, bins, per_cta, psums.as<double>(),
          pcounts.as<unsigned long long>());
      break;
    default:
      k_fold_rows<float><<<grid, FOLD_NT, smem, st>>>(o.samples.as<float>(), o.ld, n, tsamp,
                                                       period, bins, per_cta, psums.as<double>(),
                                                       pcounts.as<unsigned long long>());
      break;
  }
  PSR_CUDA(cudaGetLastError());
  k_fold_reduce<<<(unsigned)((o.nch * bins + 255) / 256), 256, 0, st>>>(
      psums.as<double>(), pcounts.as<unsigned long long>(), nparts, bins, o.nch,
      sums.as<double>(), cnts.as<unsigned long long>());
  PSR_CUDA(cudaGetLastError());
  std::vector<double> hs(o.nch * bins);
  std::vector<unsigned long long> hc(o.nch * bins);
  PSR_CUDA(cudaMemcpyAsync(hs.data(), sums.p, hs.size() * 8, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaMemcpyAsync(hc.data(), cnts.p, hc.size() * 8, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  values.resize(o.nch * bins);
  for (uint64_t i = 0; i < o.nch * bins; ++i)
    values[i] = hc[i] > 0 ? (float)(hs[i] / (double)hc[i]) : 0.0f;
  return PSR_OK;
}

int dm_response(const std::vector<float> &chp, const std::vector<double> &chmean,
                const uint32_t *d_delays, uint64_t ntrials, uint64_t nch, uint64_t bins,
                double tsamp, double period, std::vector<double> &comb, cudaStream_t st) {
  DevBuf dp, dm, dc;
  PSR_TRY(dp.ensure(chp.size() * 4));
  PSR_TRY(dm.ensure(chmean.size() * 8));
  PSR_TRY(dc.ensure(ntrials * bins * 8));
  PSR_CUDA(cudaMemcpyAsync(dp.p, chp.data(), chp.size() * 4, cudaMemcpyHostToDevice, st));
  PSR_CUDA(cudaMemcpyAsync(dm.p, chmean.data(), chmean.size() * 8, cudaMemcpyHostToDevice, st));
  k_dm_response<<<(unsigned)ntrials, 128, nch * 8, st>>>(dp.as<float>(), dm.as<double>(),
                                                         d_delays, nch, bins, tsamp, period,
                                                         dc.as<double>());
  PSR_CUDA(cudaGetLastError());
  comb.resize(ntrials * bins);
  PSR_CUDA(cudaMemcpyAsync(comb.data(), dc.p, comb.size() * 8, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  return PSR_OK;
}

}  // namespace psr
