// K3 incoherent dedispersion (dedisperse::apply, dedisperse/src/lib.rs:61-90,
// run for many trials as in the CLI loop cli/src/main.rs:462-469).
//
// out[trial][t] = sum_c data[c][t + delay[trial][c]],  t in [0, n).
//
// Integer samples (u8): every partial sum is an integer below 2^16, so the
// reference's channel-ordered f32 sum is exact and any summation order gives
// the bit-identical value.  The fast kernel stages a tile of every channel
// row into shared memory with TMA bulk copies (cp.async.bulk + mbarrier,
// double buffered), and each thread accumulates 16 consecutive samples for a
// block of trials in packed 2 x u16 lanes (samples of <= 4 bits first in
// 4 x u8 lanes, widened once per group of channels).  Consecutive trials whose
// delay for a channel is unchanged reuse the aligned sample words
// (warp-uniform test).
//
// Everything else (f32 samples, or integer sums that could exceed 2^16) uses
// a kernel that adds channels in reference order in f32.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "psr_internal.h"

namespace psr {
namespace {

constexpr int DD_NT = 256;              // threads per CTA
constexpr int DD_TPT = 16;              // samples per thread
constexpr int DD_TT = DD_NT * DD_TPT;   // samples per tile (4096)
constexpr int DD_DB = 8;                // trials per CTA (16-bit lanes only)
constexpr int DD_DB8 = 6;               // trials per CTA with 8-bit lanes (registers)
constexpr int DD_MAXCC = 32;            // rows per stage (one issuing lane each)
constexpr long long DD_SPIN_LIMIT = 1ll << 26;  // try_wait polls before a wait gives up

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false (and the error word set) if the phase never completes.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity,
                                                  unsigned *err, long long limit) {
  for (long long i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  atomicOr(err, 1u);
  return false;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

struct StageInfo {
  long long base[DD_MAXCC];    // absolute sample index of the staged row start
  int off[DD_MAXCC][DD_DB];    // tile start + delay - staged row start, per trial
};

// Issue the TMA copies of rows [c0, c0+cc) for trials [d0, d0+DB) of tile t0.
// Run by warp 0: lane i stages row c0+i.
template <int DB>
__device__ void issue_stage(const uint8_t *__restrict__ s, uint64_t ld, uint64_t ns,
                            uint64_t nch, uint64_t dstride, const uint32_t *__restrict__ delays,
                            uint64_t ntrials, uint64_t d0, uint64_t t0, uint64_t c0, int cc,
                            uint8_t *buf, int rowcap, StageInfo *info, uint64_t *bar,
                            int arm_only) {
  const int lane = threadIdx.x & 31;
  unsigned bytes = 0;
  if (lane < cc && c0 + lane < nch) {
    const uint64_t c = c0 + lane;
    uint32_t dmin = 0xffffffffu, dmax = 0;
    for (int d = 0; d < DB; ++d) {
      uint64_t tr = d0 + d < ntrials ? d0 + d : ntrials - 1;
      uint32_t v = delays[tr * dstride + c];
      dmin = min(dmin, v);
      dmax = max(dmax, v);
    }
    long long a = (long long)((t0 + dmin) & ~(uint64_t)15);
    long long rowend = (long long)((ns + 15) & ~(uint64_t)15);
    long long b = (long long)((t0 + dmax + DD_TT + 15) & ~(uint64_t)15);
    if (b > rowend) b = rowend;
    if (b > a + rowcap) b = a + rowcap;
    info->base[lane] = a;
    for (int d = 0; d < DB; ++d) {
      uint64_t tr = d0 + d < ntrials ? d0 + d : ntrials - 1;
      info->off[lane][d] = (int)((long long)t0 - a) + (int)delays[tr * dstride + c];
    }
    if (b > a) {
      bytes = (unsigned)(b - a);
      mbar_expect_tx(bar, bytes);
    }
    __syncwarp(__activemask());
    // arm_only (a test of the bounded wait): the barrier expects the bytes
    // but no copy is issued, so its phase never completes and nothing is in
    // flight when the CTA gives up.
    if (bytes && !arm_only) bulk_g2s(buf + (size_t)lane * rowcap, s + c * ld + a, bytes, bar);
  }
  __syncwarp();
  if (lane == 0) mbar_arrive(bar);
}

// BYTE_LANES: samples are at most (255 / group), so `group` channels can be
// summed in the four 8-bit lanes of a 32-bit word with a plain IADD (no lane
// overflows, so no carry crosses a byte); the byte lanes are widened into the
// 16-bit lanes once per group.  Without BYTE_LANES every channel is widened.
template <bool BYTE_LANES, int DB>
__global__ void __launch_bounds__(DD_NT, 2)
    k_dedisp_u8(const uint8_t *__restrict__ s, uint64_t ld, uint64_t ns, uint64_t nch,
                uint64_t dstride, const uint32_t *__restrict__ delays, uint64_t ntrials,
                uint64_t n, float *__restrict__ out, uint64_t ldo, double *__restrict__ part,
                uint64_t ntiles, int cc, int rowcap, int group, int accumulate, unsigned *err,
                long long spin_limit, int arm_only) {
  extern __shared__ __align__(128) uint8_t smem[];
  const size_t bstride = (size_t)cc * rowcap;  // buffer b at smem + b * bstride
  __shared__ uint64_t bars[2];
  __shared__ StageInfo info[2];
  __shared__ unsigned long long wsum[DD_NT / 32][DB];

  const uint64_t t0 = (uint64_t)blockIdx.x * DD_TT;
  const uint64_t d0 = (uint64_t)blockIdx.y * DB;
  const int tl = threadIdx.x;
  const int nchunks = (int)((nch + cc - 1) / cc);

  if (tl == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tl < 32) {
    issue_stage<DB>(s, ld, ns, nch, dstride, delays, ntrials, d0, t0, 0, cc, smem, rowcap,
                    &info[0], &bars[0], arm_only);
    if (nchunks > 1)
      issue_stage<DB>(s, ld, ns, nch, dstride, delays, ntrials, d0, t0, (uint64_t)cc, cc,
                      smem + bstride, rowcap, &info[1], &bars[1], arm_only);
  }

  uint32_t acc[DB][8];
#pragma unroll
  for (int d = 0; d < DB; ++d)
#pragma unroll
    for (int i = 0; i < 8; ++i) acc[d][i] = 0;
  uint32_t acc8[BYTE_LANES ? DB : 1][4];
#pragma unroll
  for (int d = 0; d < (BYTE_LANES ? DB : 1); ++d)
#pragma unroll
    for (int i = 0; i < 4; ++i) acc8[d][i] = 0;
  int gcount = 0;
  auto widen = [&]() {
    if constexpr (BYTE_LANES) {
#pragma unroll
      for (int d = 0; d < DB; ++d)
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          acc[d][2 * i] += __byte_perm(acc8[d][i], 0, 0x4140);
          acc[d][2 * i + 1] += __byte_perm(acc8[d][i], 0, 0x4342);
          acc8[d][i] = 0;
        }
    }
  };

  // Chunk k is staged in buffer k & 1, in that barrier's phase (k >> 1).
  // A wait that gives up ends the whole CTA: the decision is made uniform
  // by __syncthreads_or before any thread reads the buffer or reaches a
  // later barrier, so no thread is left waiting on one that left.
  int failed = -1;
  for (int k = 0; k < nchunks; ++k) {
    const int b = k & 1;
    const bool ok = mbar_wait_bounded(&bars[b], (unsigned)((k >> 1) & 1), err, spin_limit);
    if (__syncthreads_or(!ok)) {
      failed = k;
      break;
    }
    const uint64_t c0 = (uint64_t)k * cc;
    const int rows = (int)min((uint64_t)cc, (uint64_t)(nch - c0));
    const uint8_t *buf = smem + b * bstride;
    for (int r = 0; r < rows; ++r) {
      const uint4 *row16 = reinterpret_cast<const uint4 *>(buf + (size_t)r * rowcap);
      const int *offs = info[b].off[r];
      int prev = -1;
      uint32_t x0 = 0, x1 = 0, x2 = 0, x3 = 0;
#pragma unroll
      for (int d = 0; d < DB; ++d) {
        const int off = offs[d];  // shared-memory broadcast
        if (off != prev) {  // uniform across the CTA
          prev = off;
          const int q = tl + (off >> 4);
          const int o = off & 15;
          uint4 lo = row16[q], hi = row16[q + 1];
          uint32_t w0 = lo.x, w1 = lo.y, w2 = lo.z, w3 = lo.w, w4 = hi.x, w5 = hi.y, w6 = hi.z,
                   w7 = hi.w;
          if (o & 8) {
            w0 = w2; w1 = w3; w2 = w4; w3 = w5; w4 = w6; w5 = w7;
          }
          if (o & 4) {
            w0 = w1; w1 = w2; w2 = w3; w3 = w4; w4 = w5;
          }
          const unsigned sh = (unsigned)(o & 3) * 8u;
          x0 = __funnelshift_r(w0, w1, sh);
          x1 = __funnelshift_r(w1, w2, sh);
          x2 = __funnelshift_r(w2, w3, sh);
          x3 = __funnelshift_r(w3, w4, sh);
        }
        if constexpr (BYTE_LANES) {
          acc8[d][0] += x0;
          acc8[d][1] += x1;
          acc8[d][2] += x2;
          acc8[d][3] += x3;
        } else {
          acc[d][0] += __byte_perm(x0, 0, 0x4140);
          acc[d][1] += __byte_perm(x0, 0, 0x4342);
          acc[d][2] += __byte_perm(x1, 0, 0x4140);
          acc[d][3] += __byte_perm(x1, 0, 0x4342);
          acc[d][4] += __byte_perm(x2, 0, 0x4140);
          acc[d][5] += __byte_perm(x2, 0, 0x4342);
          acc[d][6] += __byte_perm(x3, 0, 0x4140);
          acc[d][7] += __byte_perm(x3, 0, 0x4342);
        }
      }
      if (BYTE_LANES && ++gcount == group) {
        widen();
        gcount = 0;
      }
    }
    __syncthreads();  // every thread is done reading buffer b
    if (tl < 32 && k + 2 < nchunks) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue_stage<DB>(s, ld, ns, nch, dstride, delays, ntrials, d0, t0, (uint64_t)(k + 2) * cc,
                      cc, smem + b * bstride, rowcap, &info[b], &bars[b], arm_only);
    }
  }
  widen();
  if (failed >= 0) {
    // Before leaving, wait (bounded) for the copies still outstanding: chunk
    // `failed` in its buffer and, if it was issued, chunk failed + 1 in the
    // other, each in the phase it was issued in.
    if (tl == 0) {
      mbar_wait_bounded(&bars[failed & 1], (unsigned)((failed >> 1) & 1), err, spin_limit);
      if (failed + 1 < nchunks)
        mbar_wait_bounded(&bars[(failed + 1) & 1], (unsigned)(((failed + 1) >> 1) & 1), err,
                          spin_limit);
    }
    return;
  }

  const uint64_t tb = t0 + (uint64_t)tl * DD_TPT;
#pragma unroll
  for (int d = 0; d < DB; ++d) {
    const uint64_t tr = d0 + d;
    float v[16];
    unsigned long long local = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      uint32_t lo = acc[d][i] & 0xffffu, hi = acc[d][i] >> 16;
      bool in0 = tb + 2 * i < n, in1 = tb + 2 * i + 1 < n;
      v[2 * i] = (float)lo;
      v[2 * i + 1] = (float)hi;
      local += (in0 ? lo : 0u) + (in1 ? hi : 0u);
    }
    if (tr < ntrials) {
      // Channel groups after the first add their (integer) partial sums to
      // the earlier groups' in f32: exact while every sum stays below 2^24.
      float *dst = out + tr * ldo + tb;
      if (tb + 16 <= n) {
        float4 *d4 = reinterpret_cast<float4 *>(dst);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          float4 w = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
          if (accumulate) {
            const float4 o = d4[i];
            w.x += o.x;
            w.y += o.y;
            w.z += o.z;
            w.w += o.w;
          }
          d4[i] = w;
        }
      } else {
        for (int i = 0; i < 16; ++i)
          if (tb + i < n) dst[i] = accumulate ? dst[i] + v[i] : v[i];
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((tl & 31) == 0) wsum[tl >> 5][d] = local;
  }
  __syncthreads();
  if (tl < DB && d0 + tl < ntrials) {
    unsigned long long t = 0;
    for (int w = 0; w < DD_NT / 32; ++w) t += wsum[w][tl];
    double *pp = &part[(d0 + tl) * ntiles + blockIdx.x];
    *pp = accumulate ? *pp + (double)t : (double)t;
  }
}

// Reference-order f32 accumulation (one output per thread per trial).
constexpr int DG_TPT = 4;
constexpr int DG_NT = 256;
constexpr int DG_TT = DG_NT * DG_TPT;
constexpr int DG_DB = 4;

template <class T>
__global__ void __launch_bounds__(DG_NT)
    k_dedisp_generic(const T *__restrict__ s, uint64_t ld, uint64_t nch,
                     const uint32_t *__restrict__ delays, uint64_t ntrials, uint64_t n,
                     float *__restrict__ out, uint64_t ldo, double *__restrict__ part,
                     uint64_t ntiles) {
  __shared__ double wsum[DG_NT / 32][DG_DB];
  __shared__ double wabs[DG_NT / 32][DG_DB];
  __shared__ int wq[DG_NT / 32][DG_DB];
  const uint64_t t0 = (uint64_t)blockIdx.x * DG_TT;
  const uint64_t d0 = (uint64_t)blockIdx.y * DG_DB;
  float acc[DG_DB][DG_TPT];
#pragma unroll
  for (int d = 0; d < DG_DB; ++d)
#pragma unroll
    for (int i = 0; i < DG_TPT; ++i) acc[d][i] = 0.0f;
  for (uint64_t c = 0; c < nch; ++c) {
    const T *row = s + c * ld;
#pragma unroll
    for (int d = 0; d < DG_DB; ++d) {
      uint64_t tr = d0 + d < ntrials ? d0 + d : ntrials - 1;
      const uint64_t dl = __ldg(&delays[tr * nch + c]);
#pragma unroll
      for (int i = 0; i < DG_TPT; ++i) {
        uint64_t t = t0 + (uint64_t)i * DG_NT + threadIdx.x;
        float v = t < n ? (float)row[t + dl] : 0.0f;
        acc[d][i] = __fadd_rn(acc[d][i], v);
      }
    }
  }
  // Non-integer samples: besides the sum, each tile records the sum of |x|
  // and the finest binary quantum among its outputs, from which
  // k_reduce_parts decides whether every partial sum is exact in f64.
  constexpr bool kFloat = std::is_same<T, float>::value;
#pragma unroll
  for (int d = 0; d < DG_DB; ++d) {
    double local = 0.0, labs = 0.0;
    int lq = kNoQuantum;
    const uint64_t tr = d0 + d;
#pragma unroll
    for (int i = 0; i < DG_TPT; ++i) {
      uint64_t t = t0 + (uint64_t)i * DG_NT + threadIdx.x;
      if (t < n) {
        if (tr < ntrials) out[tr * ldo + t] = acc[d][i];
        local += (double)acc[d][i];
        if (kFloat) {
          labs += fabs((double)acc[d][i]);
          lq = min(lq, quantum_exponent(acc[d][i]));
        }
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      local += __shfl_down_sync(0xffffffffu, local, o);
      if (kFloat) {
        labs += __shfl_down_sync(0xffffffffu, labs, o);
        lq = min(lq, __shfl_down_sync(0xffffffffu, lq, o));
      }
    }
    if ((threadIdx.x & 31) == 0) {
      wsum[threadIdx.x >> 5][d] = local;
      if (kFloat) {
        wabs[threadIdx.x >> 5][d] = labs;
        wq[threadIdx.x >> 5][d] = lq;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x < DG_DB && d0 + threadIdx.x < ntrials) {
    double t = 0.0, a = 0.0;
    int q = kNoQuantum;
    for (int w = 0; w < DG_NT / 32; ++w) {
      t += wsum[w][threadIdx.x];
      if (kFloat) {
        a += wabs[w][threadIdx.x];
        q = min(q, wq[w][threadIdx.x]);
      }
    }
    const uint64_t at = (d0 + threadIdx.x) * ntiles + blockIdx.x;
    part[at] = t;
    if (kFloat) {
      part[ntrials * ntiles + at] = a;
      part[2 * ntrials * ntiles + at] = (double)q;
    }
  }
}

// Reduction of per-tile partial sums into the series sum per trial and the
// f32 mean the FFT subtracts (search/src/lib.rs:36-40).  The reference's
// mean is a sequential f64 sum starting from -0.0.  Integer samples make
// every partial sum an exact integer below 2^53, so any order gives it.  For
// f32 samples (check = true) the tiles also recorded sum |x| and the finest
// quantum 2^q among the outputs: every partial sum, in any order, is then a
// multiple of 2^q no larger than sum |x|, so it is exact in f64 while
// sum |x| < 2^(53+q) (with a margin for the rounding of sum |x| itself).
// Otherwise the thread re-adds the trial's series sequentially, in the
// reference's order.
__global__ void k_reduce_parts(const double *part, uint64_t ntiles, uint64_t ntrials,
                               uint64_t n, double *sums, float *means, const float *series,
                               uint64_t ldo, int check) {
  uint64_t tr = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tr >= ntrials) return;
  double s = 0.0;
  for (uint64_t i = 0; i < ntiles; ++i) s += part[tr * ntiles + i];
  if (check) {
    double a = 0.0, q = (double)kNoQuantum;
    for (uint64_t i = 0; i < ntiles; ++i) {
      a += part[ntrials * ntiles + tr * ntiles + i];
      q = fmin(q, part[2 * ntrials * ntiles + tr * ntiles + i]);
    }
    const bool exact = f64_sums_exact(a, (int)q);
    if (!exact) {  // the reference's order: t = 0, 1, ..., from -0.0
      const float *x = series + tr * ldo;
      s = -0.0;
      uint64_t t = 0;
      for (; t + 4 <= n; t += 4) {  // rows start 256-byte aligned (ldo % 64 == 0)
        const float4 v = *reinterpret_cast<const float4 *>(x + t);
        s += (double)v.x;
        s += (double)v.y;
        s += (double)v.z;
        s += (double)v.w;
      }
      for (; t < n; ++t) s += (double)x[t];
    }
  }
  sums[tr] = s;
  means[tr] = (float)(s / (double)n);
}

// One CTA: the series sum and mean of launch_series_mean.
constexpr int SM_NT = 1024;
__global__ void __launch_bounds__(SM_NT)
    k_series_mean(const float *__restrict__ x, uint64_t n, double *sum_out, float *mean_out) {
  __shared__ double ss[SM_NT / 32], sa[SM_NT / 32];
  __shared__ int sq[SM_NT / 32];
  double s = 0.0, a = 0.0;
  int q = kNoQuantum;
  for (uint64_t i = threadIdx.x; i < n; i += SM_NT) {
    const float v = x[i];
    s += (double)v;
    a += fabs((double)v);
    q = min(q, quantum_exponent(v));
  }
  for (int o = 16; o; o >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, o);
    a += __shfl_down_sync(0xffffffffu, a, o);
    q = min(q, __shfl_down_sync(0xffffffffu, q, o));
  }
  if ((threadIdx.x & 31) == 0) {
    ss[threadIdx.x >> 5] = s;
    sa[threadIdx.x >> 5] = a;
    sq[threadIdx.x >> 5] = q;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  s = 0.0;
  a = 0.0;
  q = kNoQuantum;
  for (int w = 0; w < SM_NT / 32; ++w) {
    s += ss[w];
    a += sa[w];
    q = min(q, sq[w]);
  }
  if (!f64_sums_exact(a, q)) {  // the reference's order, from -0.0
    s = -0.0;
    for (uint64_t i = 0; i < n; ++i) s += (double)x[i];
  }
  if (sum_out) *sum_out = s;
  *mean_out = (float)(s / (double)n);
}

}  // namespace

int launch_series_mean(const float *d_x, uint64_t n, double *d_sum, float *d_mean,
                       cudaStream_t st) {
  k_series_mean<<<1, SM_NT, 0, st>>>(d_x, n, d_sum, d_mean);
  PSR_CUDA(cudaGetLastError());
  return PSR_OK;
}

uint64_t series_ld(uint64_t n) { return ((n + 63) / 64) * 64; }

int launch_dedisperse_ex(const DeviceObs &o, const uint32_t *d_delays, uint64_t ntrials,
                         uint64_t n, float *d_out, uint64_t ldo, double *d_part,
                         double *d_sums, float *d_means, uint64_t max_spread, unsigned *d_err,
                         cudaStream_t st, long long spin_limit, int arm_only, bool want_means) {
  const long long spin = spin_limit > 0 ? spin_limit : DD_SPIN_LIMIT;
  // Integer samples: channel groups small enough that a group's sum fits the
  // 16-bit lanes (nch * max <= 65535 when there is one group); the groups'
  // sums are added in f32, exact while the total stays below 2^24.
  const double maxv = o.kind == SAMPLE_U8 ? o.max_value() : 0.0;
  const uint64_t gch = maxv > 0.0 ? (uint64_t)(65535.0 / maxv) : 0;
  const bool packed = o.kind == SAMPLE_U8 && gch >= 1 && (double)o.nch * maxv < 16777216.0;
  if (packed) {
    const uint64_t ntiles = (n + DD_TT - 1) / DD_TT;
    int rowcap = (int)(((uint64_t)DD_TT + max_spread + 32 + 15) & ~(uint64_t)15);
    int dev = 0;
    PSR_CUDA(cudaGetDevice(&dev));
    int smax = 0;
    PSR_CUDA(cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    // two CTAs per SM: each gets half of the SM's shared memory
    int smsm = 0;
    PSR_CUDA(cudaDeviceGetAttribute(&smsm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    size_t budget = std::min((size_t)smax, (size_t)smsm / 2) - 4096;
    const uint64_t glen = std::min<uint64_t>(gch, o.nch);
    int cc = (int)std::min<uint64_t>({(uint64_t)DD_MAXCC, glen, budget / (2 * (size_t)rowcap)});
    if (cc >= 1) {
      size_t smem = 2 * (size_t)cc * rowcap;
      const int group = (int)(255.0 / maxv);
      for (uint64_t c0 = 0; c0 < o.nch; c0 += glen) {
        const uint64_t ng = std::min(glen, o.nch - c0);
        const uint8_t *sg = o.samples.as<uint8_t>() + c0 * o.ld;
        const uint32_t *dg = d_delays + c0;
        const int acc = c0 > 0 ? 1 : 0;
        const int ccg = (int)std::min<uint64_t>((uint64_t)cc, ng);
        if (group >= 2) {
          dim3 grid((unsigned)ntiles, (unsigned)((ntrials + DD_DB8 - 1) / DD_DB8));
          PSR_CUDA(cudaFuncSetAttribute(k_dedisp_u8<true, DD_DB8>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
          k_dedisp_u8<true, DD_DB8><<<grid, DD_NT, smem, st>>>(
              sg, o.ld, o.ns, ng, o.nch, dg, ntrials, n, d_out, ldo, d_part, ntiles, ccg, rowcap,
              group, acc, d_err, spin, arm_only);
        } else {
          dim3 grid((unsigned)ntiles, (unsigned)((ntrials + DD_DB - 1) / DD_DB));
          PSR_CUDA(cudaFuncSetAttribute(k_dedisp_u8<false, DD_DB>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
          k_dedisp_u8<false, DD_DB><<<grid, DD_NT, smem, st>>>(
              sg, o.ld, o.ns, ng, o.nch, dg, ntrials, n, d_out, ldo, d_part, ntiles, ccg, rowcap,
              1, acc, d_err, spin, arm_only);
        }
        PSR_CUDA(cudaGetLastError());
      }
      if (want_means) {
        k_reduce_parts<<<(unsigned)((ntrials + 127) / 128), 128, 0, st>>>(
            d_part, ntiles, ntrials, n, d_sums, d_means, d_out, ldo, 0);
        PSR_CUDA(cudaGetLastError());
      }
      return PSR_OK;
    }
  }
  const uint64_t ntiles = (n + DG_TT - 1) / DG_TT;
  dim3 grid((unsigned)ntiles, (unsigned)((ntrials + DG_DB - 1) / DG_DB));
  switch (o.kind) {
    case SAMPLE_U8:
      k_dedisp_generic<uint8_t><<<grid, DG_NT, 0, st>>>(o.samples.as<uint8_t>(), o.ld, o.nch,
                                                        d_delays, ntrials, n, d_out, ldo,
                                                        d_part, ntiles);
      break;
    case SAMPLE_U16:
      k_dedisp_generic<uint16_t><<<grid, DG_NT, 0, st>>>(o.samples.as<uint16_t>(), o.ld,
                                                         o.nch, d_delays, ntrials, n, d_out,
                                                         ldo, d_part, ntiles);
      break;
    default:
      k_dedisp_generic<float><<<grid, DG_NT, 0, st>>>(o.samples.as<float>(), o.ld, o.nch,
                                                      d_delays, ntrials, n, d_out, ldo, d_part,
                                                      ntiles);
  }
  PSR_CUDA(cudaGetLastError());
  if (want_means) {
    k_reduce_parts<<<(unsigned)((ntrials + 127) / 128), 128, 0, st>>>(
        d_part, ntiles, ntrials, n, d_sums, d_means, d_out, ldo, o.kind == SAMPLE_F32 ? 1 : 0);
    PSR_CUDA(cudaGetLastError());
  }
  return PSR_OK;
}

uint64_t dedisperse_part_count(const DeviceObs &o, uint64_t n) {
  // f32 samples: sums, sums of |x| and quanta per tile
  const uint64_t per = o.kind == SAMPLE_F32 ? 3 : 1;
  return per * std::max((n + DD_TT - 1) / DD_TT, (n + DG_TT - 1) / DG_TT);
}

}  // namespace psr
