// Gradient refinement on a folded cube: fold once, then optimise on the
// folded data.  Used by psr_refine_gradient for groups of nearby starting
// points (up to 16 of them).
//
// One pass over the filterbank folds every channel at a reference (nu_r,
// nudot_r, DM_r) into a cube C[c][s][b] (channels x subints x bins),
// channel c at its own dispersion-delayed phase
//   phi_r(c, T) = nu_r (T - tau_c) + nudot_r (T - tau_c)^2 / 2,
//   tau_c(DM) = 4148.808 DM (f_c^-2 - f_max^-2) seconds (fractional),
// with cloud-in-cell weights.  For parameters theta near the reference, the
// samples of (c, s) move in phase by d_cs = B (phi_theta(c, T_s) -
// phi_r(c, T_s)) bins, T_s the subint centre (the drift within one subint is
// neglected).  Each cube row's DFT R_cs[k] (k = 1..B/2) is taken once;
// shifting a row by d bins multiplies harmonic k by e^(-2 pi i k d / B) (a
// band-limited shift: no interpolation smoothing that would depend on the
// fractional shift), so the profile's harmonics are
//   P_k = sum_cs R_cs[k] e^(-2 pi i k d_cs / B)
// and, by Parseval, J = sum_b (p_b - mean)^2 / (n v) = sum_k w_k |P_k|^2 /
// (B n v), w_k = 2 (k < B/2), 1 (k = B/2), v = sum_c var(x_c).  Adjoint:
//   dJ/dd_cs = sum_k Re(A_k R_cs[k] e^(-2 pi i k d_cs/B) (-2 pi i k / B)),
//   A_k = 2 w_k conj(P_k) / (B n v),
//   dd_cs/dnu = B (T_s - tau_c), dd_cs/dnudot = B (T_s - tau_c)^2 / 2,
//   dd_cs/dDM = -B (nu + nudot (T_s - tau_c)) dtau_c/dDM.
// Evaluations of every candidate of a group run in the same launches.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <type_traits>
#include <vector>

#include "psr_internal.h"
#include "refine.h"

namespace psr {

// Device buffers of one cube, reused by every group of a refinement call.
struct CubeWork {
  DevBuf cube, R, chsum, tau, kc, cands, prof, g, grad;
  uint64_t rows = 0;
  double var = 1.0;
};
CubeCache::~CubeCache() { delete w; }

namespace {

constexpr double K_DM_C = 4148.808;  // dedisperse/src/lib.rs:3
constexpr int CB_NT = 256;
constexpr int CB_MAXB = 1024;

// Fold subint s of channel c (one CTA) into C[c][s][*] (the row's mean
// removed, which leaves every shifted profile's deviations unchanged and keeps
// f32 sums accurate) and the channel's sum / sum of squares.
//
// The row is cut into runs of 32 samples aligned to the global sample grid
// (rows start 64-element aligned and carry >= 64 elements of padding, so a
// run is one to eight aligned 16-byte loads that never leave the row); thread
// j folds a contiguous stretch of runs of the subint, prefetching its next run
// while it folds the current one.  Samples of a boundary run outside [t0, t1) are
// zeroed.  Phases are fixed-point fractions of a cycle (u64, 2^-64 cycle
// resolution): one CTA-wide f64 anchor at the first run, then per-thread
// offsets and per-stride advances by exact integer second differences, so no
// thread does f64 work per run.  Inside a run the bin position u (in bins)
// advances in f32; for du < 1 bin per sample the bin index is walked
// incrementally (one compare per sample), otherwise floored per sample.
// Consecutive samples of one bin are summed in registers (a0 = sum v, a1 =
// sum w v; CIC weights 1 - w and w), across run boundaries, and flushed with
// two shared-memory atomics when the bin changes.  Channel sums are integer (u8, u16) or f32
// per run (f32 data) before the f64 reduction.
constexpr int CB_RUN = 32;

template <class T>
struct RunRegs {
  static constexpr int W = (CB_RUN * (int)sizeof(T)) / 16;  // 16-byte words per run
  uint4 r[W];
};

template <class T>
__device__ __forceinline__ void load_run(const T *p, RunRegs<T> &x) {
  const uint4 *q = reinterpret_cast<const uint4 *>(p);
#pragma unroll
  for (int k = 0; k < RunRegs<T>::W; ++k) x.r[k] = __ldg(q + k);
}

__device__ __forceinline__ uint32_t word_of(const uint4 &v, int k) {
  return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

// Sample i (0..31) of a run as f32 (integer samples are exact: 2^23 + v
// assembled by a byte permute, then 2^23 subtracted).
template <class T>
__device__ __forceinline__ float run_sample(const RunRegs<T> &x, int i);
template <>
__device__ __forceinline__ float run_sample<uint8_t>(const RunRegs<uint8_t> &x, int i) {
  const uint32_t w = word_of(x.r[i >> 4], (i >> 2) & 3);
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u | (unsigned)(i & 3))) - 8388608.0f;
}
template <>
__device__ __forceinline__ float run_sample<uint16_t>(const RunRegs<uint16_t> &x, int i) {
  const uint32_t w = word_of(x.r[i >> 3], (i >> 1) & 3);
  const unsigned lo = (unsigned)(i & 1) * 2u;
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7500u | ((lo + 1u) << 4) | lo)) -
         8388608.0f;
}
template <>
__device__ __forceinline__ float run_sample<float>(const RunRegs<float> &x, int i) {
  return __uint_as_float(word_of(x.r[i >> 2], i & 3));
}

// Zero the samples of a run outside [lo, hi) (boundary runs only).
template <class T>
__device__ __forceinline__ void mask_run(RunRegs<T> &x, int lo, int hi) {
  constexpr int PER_WORD = 4 / (int)sizeof(T);
#pragma unroll
  for (int k = 0; k < RunRegs<T>::W; ++k) {
    uint32_t w[4] = {x.r[k].x, x.r[k].y, x.r[k].z, x.r[k].w};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
#pragma unroll
      for (int b = 0; b < PER_WORD; ++b) {
        const int i = (k * 4 + e) * PER_WORD + b;
        if (i < lo || i >= hi) {
          const uint32_t m = sizeof(T) == 4 ? 0xffffffffu
                                            : (((1u << (8 * sizeof(T))) - 1u) << (8 * sizeof(T) * b));
          w[e] &= ~m;
        }
      }
    }
    x.r[k] = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// Channel-sum accumulators: exact integers for 8/16-bit samples.
template <class T>
struct RunSums {
  unsigned long long s = 0, q = 0;
  __device__ __forceinline__ void add(const RunRegs<T> &x) {
    unsigned s32 = 0, q32 = 0;
#pragma unroll
    for (int k = 0; k < RunRegs<T>::W; ++k)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const uint32_t w = word_of(x.r[k], e);
        if (sizeof(T) == 1) {
          s32 = __dp4a(w, 0x01010101u, s32);
          q32 = __dp4a(w, w, q32);  // <= 32 * 255^2 per run
        } else {
          const uint32_t a = w & 0xffffu, b = w >> 16;
          s32 += a + b;
          q += (unsigned long long)(a * a) + (unsigned long long)(b * b);
        }
      }
    s += s32;
    q += q32;
  }
  // One 16-byte chunk (staged tiles).
  __device__ __forceinline__ void add_chunk(const uint4 &v) {
    unsigned s32 = 0, q32 = 0;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const uint32_t w = word_of(v, e);
      if (sizeof(T) == 1) {
        s32 = __dp4a(w, 0x01010101u, s32);
        q32 = __dp4a(w, w, q32);
      } else {
        const uint32_t a = w & 0xffffu, b = w >> 16;
        s32 += a + b;
        q += (unsigned long long)(a * a) + (unsigned long long)(b * b);
      }
    }
    s += s32;
    q += q32;
  }
  __device__ __forceinline__ double sum() const { return (double)s; }
  __device__ __forceinline__ double sq() const { return (double)q; }
};
template <>
struct RunSums<float> {
  double s = 0.0, q = 0.0;
  __device__ __forceinline__ void add(const RunRegs<float> &x) {
    float ps = 0.0f, pq = 0.0f;
#pragma unroll
    for (int i = 0; i < CB_RUN; ++i) {
      const float v = run_sample<float>(x, i);
      ps += v;
      pq = fmaf(v, v, pq);
    }
    s += (double)ps;
    q += (double)pq;
  }
  __device__ __forceinline__ void add_chunk(const uint4 &v) {
    float ps = 0.0f, pq = 0.0f;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float x = __uint_as_float(word_of(v, e));
      ps += x;
      pq = fmaf(x, x, pq);
    }
    s += (double)ps;
    q += (double)pq;
  }
  __device__ __forceinline__ double sum() const { return s; }
  __device__ __forceinline__ double sq() const { return q; }
};

// frac(x) as a u64 fraction of a cycle.
__device__ __forceinline__ unsigned long long fix_frac(double x) {
  const double f = x - floor(x);
  return __double2ull_rz(ldexp(f, 64));
}

// Bin accumulators of one CTA.  PrivateBins: one column per thread,
// h[b * nt + tid] (bank = tid mod 32 for every b: no conflicts, no atomics),
// summed over threads at the end; for (B + 1) * threads <= CB_PRIV floats.
// SharedBins: one row updated with shared-memory atomics (large B).
constexpr int CB_PRIV = 8448;  // 33 KB: 64 threads at B = 128
// Both carry B + 1 rows: add2 puts a sample's second cloud-in-cell share in
// row b + 1 without wrapping, and row B is folded into row 0 at the end.
struct PrivateBins {
  float *h;  // this thread's column: h[b * nt]
  int nt;
  __device__ __forceinline__ void add(int b, float x) const { h[b * nt] += x; }
  __device__ __forceinline__ void add2(int b, float x0, float x1) const {
    float *p = h + b * nt;
    p[0] += x0;
    p[nt] += x1;
  }
};
struct SharedBins {
  float *h;
  __device__ __forceinline__ void add(int b, float x) const { atomicAdd(&h[b], x); }
  __device__ __forceinline__ void add2(int b, float x0, float x1) const {
    atomicAdd(&h[b], x0);
    atomicAdd(&h[b + 1], x1);
  }
};

template <class Bins>
__device__ __forceinline__ void flush_bins(const Bins &bins, int bin, int B, float a0, float a1) {
  bins.add(bin, a0 - a1);
  bins.add(bin + 1 == B ? 0 : bin + 1, a1);
}

// Open bin of a thread's walk: samples of bin `bin` summed so far (a0 = sum
// v, a1 = sum w v); bin < 0 when nothing is open.
struct OpenBin {
  int bin = -1;
  float a0 = 0.0f, a1 = 0.0f;
  template <class Bins>
  __device__ __forceinline__ void move_to(int b, const Bins &bins, int B) {
    if (b != bin) {
      if (bin >= 0) flush_bins(bins, bin, B, a0, a1);
      bin = b;
      a0 = a1 = 0.0f;
    }
  }
};

// du >= 1 bin per sample: every sample starts a new bin, so each goes
// straight to its two bins (the open bin, if any, is flushed first).
template <class T, class Bins>
__device__ __forceinline__ void scatter_run(const RunRegs<T> &x, float u, float du, int B,
                                            const Bins &bins, OpenBin &ob) {
  if (ob.bin >= 0) {
    flush_bins(bins, ob.bin, B, ob.a0, ob.a1);
    ob.bin = -1;
    ob.a0 = ob.a1 = 0.0f;
  }
  const float fB = (float)B;
#pragma unroll
  for (int i = 0; i < CB_RUN; ++i) {
    // 0 <= u < B here (u >= B is wrapped below and at run starts), so
    // floor(u) <= B - 1 and its second share lands in rows 1..B
    const float v = run_sample<T>(x, i);
    const float fl = floorf(u);
    const float wv = (u - fl) * v;
    bins.add2((int)fl, v - wv, wv);
    u += du;
    if (u >= fB) u -= fB;
  }
}

// Fold one run starting at bin position u (bins) advancing du per sample;
// the open bin carries over from the previous run of the same thread.
template <class T, class Bins>
__device__ __forceinline__ void fold_run(const RunRegs<T> &x, float u, float du, int B,
                                         const Bins &bins, OpenBin &ob, RunSums<T> &sums) {
  sums.add(x);
  if (du < 1.0f) {
    int b = (int)u;
    if (b >= B) b = 0, u = 0.0f;
    float w = u - (float)b;
    ob.move_to(b, bins, B);
#pragma unroll
    for (int i = 0; i < CB_RUN; ++i) {
      const float v = run_sample<T>(x, i);
      ob.a0 += v;
      ob.a1 = fmaf(w, v, ob.a1);
      w += du;
      if (w >= 1.0f) {
        flush_bins(bins, ob.bin, B, ob.a0, ob.a1);
        ob.bin = ob.bin + 1 == B ? 0 : ob.bin + 1;
        w -= 1.0f;
        ob.a0 = ob.a1 = 0.0f;
      }
    }
  } else {
    scatter_run(x, u, du, B, bins, ob);
  }
}

// 8-bit runs: a run that stays inside one bin (or crosses one bin edge) is
// folded from two integer sums instead of sample by sample.  With w_i = w0 +
// i du the run adds sum (1 - w_i) v_i and sum w_i v_i to bins b and b + 1,
// i.e. a0 += S and a1 += w0 S + du T with S = sum v_i, T = sum i v_i (dp4a
// over the packed bytes, exact); a run whose w reaches 1 at sample p is split
// there (byte-masked dp4a for the prefix).  Runs with more crossings (du >=
// 1/31 bins per sample) take the sample-by-sample walk.
__device__ __forceinline__ uint32_t prefix_mask(int p, int k) {
  const int cnt = min(max(p - 4 * k, 0), 4);
  return cnt == 0 ? 0u : (0xffffffffu >> (32 - 8 * cnt));
}

template <class Bins>
__device__ __forceinline__ void fold_run(const RunRegs<uint8_t> &x, float u, float du, int B,
                                         const Bins &bins, OpenBin &ob,
                                         RunSums<uint8_t> &sums) {
  // S = sum v, Q = sum v^2 (the channel statistics), T = sum i v.
  unsigned S = 0, Q = 0, T = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const uint32_t wd = word_of(x.r[k >> 2], k & 3);
    S = __dp4a(wd, 0x01010101u, S);
    Q = __dp4a(wd, wd, Q);
    T = __dp4a(wd, 0x03020100u + 0x04040404u * (unsigned)k, T);
  }
  sums.s += S;
  sums.q += Q;
  int b = (int)u;
  if (b >= B) b = 0, u = 0.0f;
  const float w0 = u - (float)b;
  const float wend = fmaf(31.0f, du, w0);
  if (du < 1.0f && wend < 2.0f) {
    ob.move_to(b, bins, B);
    if (wend < 1.0f) {
      ob.a0 += (float)S;
      ob.a1 += fmaf(w0, (float)S, du * (float)T);
      return;
    }
    // first sample with w >= 1 (the walk's rule, with its f32 rounding)
    int p = min(max((int)ceilf((1.0f - w0) / du), 1), 31);
    if (fmaf((float)(p - 1), du, w0) >= 1.0f) --p;
    else if (fmaf((float)p, du, w0) < 1.0f) ++p;
    unsigned S1 = 0, T1 = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const uint32_t wd = word_of(x.r[k >> 2], k & 3) & prefix_mask(p, k);
      S1 = __dp4a(wd, 0x01010101u, S1);
      T1 = __dp4a(wd, 0x03020100u + 0x04040404u * (unsigned)k, T1);
    }
    const float s1 = (float)S1, t1 = (float)T1, s2 = (float)(S - S1), t2 = (float)(T - T1);
    flush_bins(bins, ob.bin, B, ob.a0 + s1, ob.a1 + fmaf(w0, s1, du * t1));
    ob.bin = ob.bin + 1 == B ? 0 : ob.bin + 1;
    ob.a0 = s2;
    ob.a1 = fmaf(w0 - 1.0f, s2, du * t2);
    return;
  }
  // Sample-by-sample walk.
  if (du < 1.0f) {
    float w = w0;
    ob.move_to(b, bins, B);
#pragma unroll
    for (int i = 0; i < CB_RUN; ++i) {
      const float v = run_sample<uint8_t>(x, i);
      ob.a0 += v;
      ob.a1 = fmaf(w, v, ob.a1);
      w += du;
      if (w >= 1.0f) {
        flush_bins(bins, ob.bin, B, ob.a0, ob.a1);
        ob.bin = ob.bin + 1 == B ? 0 : ob.bin + 1;
        w -= 1.0f;
        ob.a0 = ob.a1 = 0.0f;
      }
    }
  } else {
    scatter_run(x, u, du, B, bins, ob);
  }
}

// PRIV: per-thread bin columns in dynamic shared memory (B * blockDim.x
// floats); otherwise one shared row with atomics.  blockDim.x is a multiple
// of 32, at most CB_NT.
template <class T, bool PRIV>
__global__ void __launch_bounds__(CB_NT)
    k_cube_fold(const T *__restrict__ x, uint64_t ld, uint64_t n, int S, int B, double tsamp,
                double nu, double nudot, const double *__restrict__ tau,
                float *__restrict__ cube, double *__restrict__ chsum) {
  extern __shared__ float hist[];
  __shared__ unsigned long long fx[5];
  __shared__ double red[2][CB_NT / 32];
  __shared__ float mean_s;
  const int nt = (int)blockDim.x, tid = (int)threadIdx.x;
  const int s = blockIdx.x;
  const uint64_t c = blockIdx.y;
  const int hn = PRIV ? (B + 1) * nt : B + 1;
  for (int i = tid; i < hn; i += nt) hist[i] = 0.0f;
  const uint64_t t0 = (n * (uint64_t)s) / (uint64_t)S, t1 = (n * (uint64_t)(s + 1)) / (uint64_t)S;
  const uint64_t rlo = t0 / CB_RUN, rhi = (t1 + CB_RUN - 1) / CB_RUN;  // runs [rlo, rhi)
  if (tid == 0) {
    // Phase (cycles) at sample m of the channel: nu td + nudot td^2 / 2,
    // td = m tsamp - tau_c; f = d phase / d sample, g = d f / d sample.
    const double td = (double)(rlo * CB_RUN) * tsamp - tau[c];
    const double f = (nu + nudot * td) * tsamp, g = nudot * tsamp * tsamp;
    const double R = (double)CB_RUN;
    fx[0] = fix_frac(nu * td + 0.5 * nudot * td * td);  // phase at the first run
    fx[1] = fix_frac(f);                                // cycles/sample there
    fx[2] = fix_frac(R * f + 0.5 * g * R * R);          // run 1 - run 0
    fx[3] = fix_frac(g * R * R);                        // its change per run
    fx[4] = fix_frac(g * R);                            // f change per run
  }
  __syncthreads();
  // Thread j folds the contiguous runs [rlo + j q, rlo + (j + 1) q) so that
  // the open bin carries from run to run.  Phase at run m (from rlo):
  // P0 + m d1 + m (m - 1) / 2 d2, exact modulo 1.
  const uint64_t q = (rhi - rlo + nt - 1) / nt;
  const unsigned long long m = (unsigned long long)tid * q;
  unsigned long long P = fx[0] + m * fx[2] + (m * (m - 1) / 2) * fx[3];
  unsigned long long A = fx[2] + m * fx[3];
  unsigned long long F = fx[1] + m * fx[4];
  const unsigned long long D2 = fx[3], G = fx[4];
  const float Bs = (float)B * 5.42101086242752217e-20f;  // B 2^-64
  const float fB = (float)B;
  const T *row = x + c * ld;
  typename std::conditional<PRIV, PrivateBins, SharedBins>::type bins;
  if constexpr (PRIV) bins = PrivateBins{hist + tid, nt};
  else bins = SharedBins{hist};
  RunSums<T> sums;
  OpenBin ob;
  const uint64_t r0 = rlo + m;
  const int cnt = r0 < rhi ? (int)(min(r0 + q, rhi) - r0) : 0;
  // Only the subint's first and last runs can hold samples outside [t0, t1).
  const int lo0 = (int)(t0 - rlo * CB_RUN), hi1 = (int)(t1 - (rhi - 1) * CB_RUN);
  const bool has_first = r0 == rlo, has_last = r0 + (uint64_t)cnt == rhi;
  const T *src = row + r0 * CB_RUN;
  RunRegs<T> cur, nxt;
  if (cnt > 0) load_run(src, cur);
  for (int i = 0; i < cnt; ++i) {
    if (i + 1 < cnt) load_run(src + (i + 1) * CB_RUN, nxt);
    if ((has_first && i == 0 && lo0 != 0) || (has_last && i == cnt - 1 && hi1 != CB_RUN))
      mask_run(cur, (has_first && i == 0) ? lo0 : 0, (has_last && i == cnt - 1) ? hi1 : CB_RUN);
    float u = __ull2float_rn(P) * Bs;
    if (u >= fB) u -= fB;
    fold_run(cur, u, __ull2float_rn(F) * Bs, B, bins, ob, sums);
    P += A;
    A += D2;
    F += G;
    cur = nxt;
  }
  if (ob.bin >= 0) flush_bins(bins, ob.bin, B, ob.a0, ob.a1);
  double sum = sums.sum(), sq = sums.sq();
  for (int o = 16; o; o >>= 1) {
    sum += __shfl_down_sync(0xffffffffu, sum, o);
    sq += __shfl_down_sync(0xffffffffu, sq, o);
  }
  if ((tid & 31) == 0) {
    red[0][tid >> 5] = sum;
    red[1][tid >> 5] = sq;
  }
  __syncthreads();
  if (tid < 2) {
    double a = 0.0;
    for (int w2 = 0; w2 < nt / 32; ++w2) a += red[tid][w2];
    chsum[(c * (uint64_t)S + (uint64_t)s) * 2 + tid] = a;
    if (tid == 0) mean_s = (float)(a / (double)B);
  }
  __syncthreads();
  float *dst = cube + (c * (uint64_t)S + (uint64_t)s) * (uint64_t)B;
  for (int b = tid; b < B; b += nt) {
    float v;
    if constexpr (PRIV) {
      // row sums (row B joins row 0), skewed by the thread index so that a
      // warp's reads of 32 consecutive rows fall in 32 different banks
      v = 0.0f;
      for (int r = b; r <= B; r += B) {
        const float *hb = hist + r * nt;
        for (int t = 0; t < nt; ++t) {
          int k = t + tid;
          if (k >= nt) k -= nt;
          v += hb[k];
        }
        if (b != 0) break;
      }
    } else {
      v = hist[b] + (b == 0 ? hist[B] : 0.0f);
    }
    dst[b] = v - mean_s;
  }
}

// Bin-owner fold for 1/31 <= du < 1 bins per sample (each bin holds 1 to 31
// consecutive samples per period).  Each warp stages tiles of CB_TL samples
// of the subint in shared memory; lane l owns bins l, l + 32, ... < B and,
// for every unwrapped bin index m = b + k B that the tile's phase range
// crosses, gathers the samples i in [Q(m), Q(m + 1)), Q(m) = ceil((m - ua) /
// du) clamped to the tile (ua = bin position of the tile's first sample, the
// phase linear across the tile).  Adjacent bins use the same Q, so every
// sample is counted once.  The lane keeps S_b = sum v and T_b = sum (u - m) v
// in registers; at the end bin b of the cloud-in-cell fold is S_b - T_b +
// T_(b-1).  No atomics, no per-sample branches.
constexpr int CB_TL = 2048;
constexpr int CB_BO_MAXB = 256;
constexpr int CB_BO_NB = CB_BO_MAXB / 32;

template <class T>
__global__ void __launch_bounds__(CB_NT)
    k_cube_fold_bo(const T *__restrict__ x, uint64_t ld, uint64_t n, int S, int B, double tsamp,
                   double nu, double nudot, const double *__restrict__ tau,
                   float *__restrict__ cube, double *__restrict__ chsum) {
  extern __shared__ __align__(16) unsigned char smem_bo[];
  T *tiles = reinterpret_cast<T *>(smem_bo);  // [warp][CB_TL]
  float *wS = reinterpret_cast<float *>(smem_bo + (size_t)(CB_NT / 32) * CB_TL * sizeof(T));
  float *wT = wS + (CB_NT / 32) * B;
  __shared__ unsigned long long fx[5];
  __shared__ double red[2][CB_NT / 32];
  __shared__ float mean_s;
  const int tid = (int)threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int s = blockIdx.x;
  const uint64_t c = blockIdx.y;
  const uint64_t t0 = (n * (uint64_t)s) / (uint64_t)S, t1 = (n * (uint64_t)(s + 1)) / (uint64_t)S;
  const uint64_t k0 = t0 / CB_TL, k1 = (t1 + CB_TL - 1) / CB_TL;  // tiles [k0, k1)
  if (tid == 0) {
    const double td = (double)(k0 * CB_TL) * tsamp - tau[c];
    const double f = (nu + nudot * td) * tsamp, g = nudot * tsamp * tsamp;
    const double L = (double)CB_TL;
    fx[0] = fix_frac(nu * td + 0.5 * nudot * td * td);  // phase at tile k0
    fx[1] = fix_frac(f);                                // cycles/sample there
    fx[2] = fix_frac(L * f + 0.5 * g * L * L);          // tile 1 - tile 0
    fx[3] = fix_frac(g * L * L);                        // its change per tile
    fx[4] = fix_frac(g * L);                            // f change per tile
  }
  __syncthreads();
  const float Bs = (float)B * 5.42101086242752217e-20f;  // B 2^-64
  const float fB = (float)B;
  const T *row = x + c * ld;
  T *tile = tiles + (size_t)warp * CB_TL;
  float Sb[CB_BO_NB], Tb[CB_BO_NB];
#pragma unroll
  for (int j = 0; j < CB_BO_NB; ++j) Sb[j] = Tb[j] = 0.0f;
  RunSums<T> sums;
  constexpr int PER = 16 / (int)sizeof(T);  // samples per 16-byte chunk
  for (uint64_t k = k0 + warp; k < k1; k += CB_NT / 32) {
    const uint64_t ta = k * CB_TL;
    // Stage the tile (chunks wholly outside [t0, t1) are not loaded).
    for (int q = lane; q < CB_TL / PER; q += 32) {
      const uint64_t cs = ta + (uint64_t)q * PER;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (cs < t1 && cs + PER > t0) {
        v = __ldg(reinterpret_cast<const uint4 *>(row + cs));
        if (cs < t0 || cs + PER > t1) {  // mask samples outside [t0, t1)
          T e[PER];
          memcpy(e, &v, 16);
#pragma unroll
          for (int u = 0; u < PER; ++u)
            if (cs + u < t0 || cs + u >= t1) e[u] = (T)0;
          memcpy(&v, e, 16);
        }
      }
      reinterpret_cast<uint4 *>(tile)[q] = v;
      sums.add_chunk(v);
    }
    __syncwarp();
    // Phase of the tile: fixed-point at its first sample, linear across it.
    const unsigned long long kk = k - k0;
    const unsigned long long P = fx[0] + kk * fx[2] + (kk * (kk - 1) / 2) * fx[3];
    const unsigned long long F = fx[1] + kk * fx[4];
    float ua = __ull2float_rn(P) * Bs;
    if (ua >= fB) ua -= fB;
    // (a tile's du only departs from the launch's nominal 1/31..1 through
    // nudot; the floor keeps the partition finite)
    const float du = fmaxf(__ull2float_rn(F) * Bs, 1e-3f);
    const float inv = 1.0f / du;
    const float uend = fmaf((float)CB_TL, du, ua);  // unwrapped phase past the tile
    // an interval of 1/du holds at most floor(1/du) + 1 samples; one more
    // covers the rounding of Q
    const int cmax = (int)inv + 2;
    const int mfirst = (int)ua;  // bin of the tile's first sample
#pragma unroll
    for (int j = 0; j < CB_BO_NB; ++j) {
      const int b = lane + 32 * j;
      if (b >= B) break;
      // first unwrapped m = b + k B >= mfirst (0 <= mfirst < B)
      int m = b >= mfirst ? b : b + B;
      float sj = 0.0f, tj = 0.0f;
      for (; (float)m < uend; m += B) {
        const int i0 = max(0, (int)ceilf(((float)m - ua) * inv));
        const int i1 = min(CB_TL, (int)ceilf(((float)(m + 1) - ua) * inv));
        // sum v and sum (i - i0) v of the bin's samples, then its weights
        // w_i = w_0 + (i - i0) du, w_0 = ua + i0 du - m
        float sl = 0.0f, il = 0.0f, fq = 0.0f;
        for (int q = 0; q < cmax; ++q) {
          if (i0 + q >= i1) break;
          const float v = (float)tile[i0 + q];
          sl += v;
          il = fmaf(fq, v, il);
          fq += 1.0f;
        }
        sj += sl;
        tj = fmaf(fmaf((float)i0, du, ua) - (float)m, sl, fmaf(du, il, tj));
      }
      Sb[j] += sj;
      Tb[j] += tj;
    }
    __syncwarp();
  }
  // Per-warp bin sums to shared memory, then across warps.
#pragma unroll
  for (int j = 0; j < CB_BO_NB; ++j) {
    const int b = lane + 32 * j;
    if (b < B) {
      wS[warp * B + b] = Sb[j];
      wT[warp * B + b] = Tb[j];
    }
  }
  double sum = sums.sum(), sq = sums.sq();
  for (int o = 16; o; o >>= 1) {
    sum += __shfl_down_sync(0xffffffffu, sum, o);
    sq += __shfl_down_sync(0xffffffffu, sq, o);
  }
  if (lane == 0) {
    red[0][warp] = sum;
    red[1][warp] = sq;
  }
  __syncthreads();
  if (tid < 2) {
    double a = 0.0;
    for (int w2 = 0; w2 < CB_NT / 32; ++w2) a += red[tid][w2];
    chsum[(c * (uint64_t)S + (uint64_t)s) * 2 + tid] = a;
    if (tid == 0) mean_s = (float)(a / (double)B);
  }
  __syncthreads();
  float *dst = cube + (c * (uint64_t)S + (uint64_t)s) * (uint64_t)B;
  for (int b = tid; b < B; b += CB_NT) {
    const int bp = b == 0 ? B - 1 : b - 1;
    float sb = 0.0f, tb = 0.0f, tp = 0.0f;
    for (int w2 = 0; w2 < CB_NT / 32; ++w2) {
      sb += wS[w2 * B + b];
      tb += wT[w2 * B + b];
      tp += wT[w2 * B + bp];
    }
    dst[b] = sb - tb + tp - mean_s;
  }
}

// Threads per fold CTA for B bins: private columns when (B + 1) * threads fits
// CB_PRIV floats with at least 32 threads.
int cube_fold_threads(int B, bool &priv) {
  int nt = (CB_PRIV / (B + 1)) / 32 * 32;
  priv = nt >= 32;
  return priv ? std::min(nt, CB_NT) : CB_NT;
}

// du = bins per sample at the reference: the bin-owner gather for 1/31 <= du
// < 1 (B <= 256), otherwise runs (analytic for 8-bit data at du < 1/31,
// walked or scattered otherwise).
template <class T>
int launch_cube_fold(dim3 grid, int B, cudaStream_t st, const T *x, uint64_t ld, uint64_t n,
                     int S, double tsamp, double nu, double nudot, const double *tau,
                     float *cube, double *chsum) {
  const double du = nu * tsamp * (double)B;
  if (du >= 1.0 / 31.0 && du < 1.0 && B <= CB_BO_MAXB) {
    const size_t sm = (size_t)(CB_NT / 32) * CB_TL * sizeof(T) + (size_t)2 * (CB_NT / 32) * B * 4;
    PSR_CUDA(cudaFuncSetAttribute(k_cube_fold_bo<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sm));
    k_cube_fold_bo<T><<<grid, CB_NT, sm, st>>>(x, ld, n, S, B, tsamp, nu, nudot, tau, cube,
                                              chsum);
    return PSR_OK;
  }
  // Below 1/31 bins per sample runs rarely change bin: one shared row with
  // 256 threads; above 1 every sample changes bin: private columns.
  bool priv = false;
  const int nt = du < 1.0 ? CB_NT : cube_fold_threads(B, priv);
  if (priv)
    k_cube_fold<T, true><<<grid, nt, (size_t)(B + 1) * nt * 4, st>>>(
        x, ld, n, S, B, tsamp, nu, nudot, tau, cube, chsum);
  else
    k_cube_fold<T, false><<<grid, nt, (size_t)(B + 1) * 4, st>>>(x, ld, n, S, B, tsamp, nu,
                                                                nudot, tau, cube, chsum);
  return PSR_OK;
}

struct CandDev {
  double nu, nudot, dm;
};

__device__ __forceinline__ double cube_shift(const CandDev &q, double nu_r, double nudot_r,
                                             double dm_r, double Ts, double kc, double B,
                                             double &tdq) {
  const double taur = kc * dm_r, tauq = kc * q.dm;
  const double tdr = Ts - taur;
  tdq = Ts - tauq;
  const double phr = nu_r * tdr + 0.5 * nudot_r * tdr * tdr;
  const double phq = q.nu * tdq + 0.5 * q.nudot * tdq * tdq;
  return (phq - phr) * B;
}

// Shift of row r = (c, s) for a candidate, in bins, and T_s - tau_c(DM).
__device__ __forceinline__ double row_shift(const CandDev &q, double nu_r, double nudot_r,
                                            double dm_r, double Tsub, const double *kc, int S,
                                            int B, uint64_t r, double &tdq, double &kcc) {
  const uint64_t c = r / (uint64_t)S;
  const int s = (int)(r % (uint64_t)S);
  const double Ts = ((double)s + 0.5) * Tsub;
  kcc = kc[c];
  return cube_shift(q, nu_r, nudot_r, dm_r, Ts, kcc, (double)B, tdq);
}

// R[r][k-1] = sum_b C[r][b] e^(-2 pi i k b / B), k = 1..B/2; one CTA per
// CB_ROWS rows, twiddles from a shared table.
constexpr int CB_ROWS = 32;
__global__ void __launch_bounds__(CB_NT)
    k_cube_dft(const float *__restrict__ cube, uint64_t rows, int B, float2 *__restrict__ R) {
  __shared__ float2 tw[CB_MAXB];
  __shared__ float row[CB_MAXB];
  for (int m = threadIdx.x; m < B; m += blockDim.x) {
    float sn, cs;
    sincospif(-2.0f * (float)m / (float)B, &sn, &cs);
    tw[m] = make_float2(cs, sn);
  }
  const int K = B / 2;
  const uint64_t r1 = min((uint64_t)(blockIdx.x + 1) * CB_ROWS, rows);
  for (uint64_t r = (uint64_t)blockIdx.x * CB_ROWS; r < r1; ++r) {
    __syncthreads();
    for (int b = threadIdx.x; b < B; b += blockDim.x) row[b] = cube[r * (uint64_t)B + b];
    __syncthreads();
    for (int k = threadIdx.x + 1; k <= K; k += blockDim.x) {
      float re = 0.0f, im = 0.0f;
      int m = 0;
      for (int b = 0; b < B; ++b) {
        const float2 w = tw[m];
        re += row[b] * w.x;
        im += row[b] * w.y;
        m += k;
        if (m >= B) m -= B;
      }
      R[r * (uint64_t)K + (k - 1)] = make_float2(re, im);
    }
  }
}

// P[cand][k] for every candidate: CTA (chunk of rows, candidate); thread k
// accumulates its harmonic over the chunk's rows, then one f64 atomic pair.
__global__ void __launch_bounds__(CB_NT)
    k_cube_harmonics(const float2 *__restrict__ R, uint64_t rows, int S, int B,
                     const double *__restrict__ kc, double Tsub, double nu_r, double nudot_r,
                     double dm_r, const CandDev *__restrict__ cands, int rows_per_cta,
                     double *__restrict__ P) {
  __shared__ float dsh[CB_NT];  // shift / B, reduced to [0, 1)
  const int k = blockIdx.y;
  const CandDev q = cands[k];
  const int K = B / 2;
  const uint64_t r0 = (uint64_t)blockIdx.x * rows_per_cta;
  const int nr = (int)min((uint64_t)rows_per_cta, rows - r0);
  if (threadIdx.x < nr) {
    double tdq, kcc;
    const double d = row_shift(q, nu_r, nudot_r, dm_r, Tsub, kc, S, B, r0 + threadIdx.x, tdq,
                               kcc) / (double)B;
    dsh[threadIdx.x] = (float)(d - floor(d));
  }
  __syncthreads();
  for (int h = threadIdx.x + 1; h <= K; h += blockDim.x) {
    float re = 0.0f, im = 0.0f;
    for (int i = 0; i < nr; ++i) {
      // e^(-2 pi i h d) with h d reduced mod 1 in f32
      float x = (float)h * dsh[i];
      x -= floorf(x);
      float sn, cs;
      sincospif(-2.0f * x, &sn, &cs);
      const float2 v = R[(r0 + i) * (uint64_t)K + (h - 1)];
      re += v.x * cs - v.y * sn;
      im += v.x * sn + v.y * cs;
    }
    atomicAdd(&P[((uint64_t)k * K + (h - 1)) * 2], (double)re);
    atomicAdd(&P[((uint64_t)k * K + (h - 1)) * 2 + 1], (double)im);
  }
}

// Gradient: each warp takes 32 rows at a time; lane l computes row l's shift
// (the only f64 work), then the warp walks the 32 rows with the lanes
// splitting each row's harmonics.
__global__ void __launch_bounds__(CB_NT)
    k_cube_grad(const float2 *__restrict__ R, uint64_t rows, int S, int B,
                const double *__restrict__ kc, double Tsub, double nu_r, double nudot_r,
                double dm_r, const CandDev *__restrict__ cands, const float2 *__restrict__ A,
                double *__restrict__ grad) {
  __shared__ double red[3][CB_NT / 32];
  const int k = blockIdx.y;
  const CandDev q = cands[k];
  const int K = B / 2;
  const float2 *Ak = A + (uint64_t)k * K;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t nwarps = (uint64_t)gridDim.x * (CB_NT / 32);
  const float twopi_b = 6.283185307179586f / (float)B;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  for (uint64_t r0 = ((uint64_t)blockIdx.x * (CB_NT / 32) + warp) * 32; r0 < rows;
       r0 += nwarps * 32) {
    const uint64_t rl = r0 + lane;
    double tdq = 0.0, kcc = 0.0;
    float dl = 0.0f;
    if (rl < rows) {
      const double dd = row_shift(q, nu_r, nudot_r, dm_r, Tsub, kc, S, B, rl, tdq, kcc) /
                        (double)B;
      dl = (float)(dd - floor(dd));
    }
    float gl = 0.0f;  // this lane's row's dJ/dd, assembled below
    const int nr = (int)min((uint64_t)32, rows - r0);
    for (int i = 0; i < nr; ++i) {
      const float d = __shfl_sync(0xffffffffu, dl, i);
      const float2 *Rr = R + (r0 + i) * (uint64_t)K;
      float g = 0.0f;
      for (int h = lane + 1; h <= K; h += 32) {
        float x = (float)h * d;
        x -= floorf(x);
        float sn, cs;
        sincospif(-2.0f * x, &sn, &cs);
        const float2 v = Rr[h - 1];
        // z = R e^(-2 pi i h d) (-2 pi i h / B); contribution Re(A_h z)
        const float zr = v.x * cs - v.y * sn, zi = v.x * sn + v.y * cs;
        const float f = twopi_b * (float)h;
        const float2 a = Ak[h - 1];
        g += a.x * (zi * f) - a.y * (-zr * f);
      }
      for (int o = 16; o; o >>= 1) g += __shfl_xor_sync(0xffffffffu, g, o);
      if (lane == i) gl = g;
    }
    if (rl < rows) {
      const double Bd = (double)B, gg = (double)gl;
      a0 += gg * Bd * tdq;
      a1 += gg * Bd * 0.5 * tdq * tdq;
      a2 += gg * (-Bd * (q.nu + q.nudot * tdq) * kcc);
    }
  }
  for (int o = 16; o; o >>= 1) {
    a0 += __shfl_xor_sync(0xffffffffu, a0, o);
    a1 += __shfl_xor_sync(0xffffffffu, a1, o);
    a2 += __shfl_xor_sync(0xffffffffu, a2, o);
  }
  if (lane == 0) {
    red[0][warp] = a0;
    red[1][warp] = a1;
    red[2][warp] = a2;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double x = 0.0;
    for (int w = 0; w < CB_NT / 32; ++w) x += red[threadIdx.x][w];
    atomicAdd(&grad[(uint64_t)k * 3 + threadIdx.x], x);
  }
}


// v = sum over channels of each channel's sample variance (the variance of a
// sum of independent channels), from the per-(channel, subint) sums.
__global__ void __launch_bounds__(CB_NT)
    k_cube_var(const double *__restrict__ chsum, uint64_t nch, int S, uint64_t n,
               double *__restrict__ out) {
  __shared__ double red[CB_NT / 32];
  double v = 0.0;
  for (uint64_t c = threadIdx.x; c < nch; c += CB_NT) {
    double s1 = 0.0, s2 = 0.0;
    for (int s = 0; s < S; ++s) {
      s1 += chsum[(c * S + s) * 2];
      s2 += chsum[(c * S + s) * 2 + 1];
    }
    const double m = s1 / (double)n;
    v += fmax(s2 / (double)n - m * m, 0.0);
  }
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    for (int w = 0; w < CB_NT / 32; ++w) a += red[w];
    out[0] = a;
  }
}

int build_cube(const DeviceObs &o, uint64_t n, int S, int B, double nu, double nudot, double dm,
               CubeWork &w, cudaStream_t st) {
  const uint64_t nch = o.nch;
  double fmax = 0.0;
  for (uint64_t c = 0; c < nch; ++c) fmax = std::fmax(fmax, o.h.fch1 + (double)c * o.h.foff);
  std::vector<double> kc(nch), tau(nch);
  for (uint64_t c = 0; c < nch; ++c) {
    const double f = o.h.fch1 + (double)c * o.h.foff;
    kc[c] = K_DM_C * (1.0 / (f * f) - 1.0 / (fmax * fmax));
    tau[c] = kc[c] * dm;
  }
  w.rows = nch * (uint64_t)S;
  PSR_TRY(w.cube.ensure(w.rows * B * 4));
  PSR_TRY(w.chsum.ensure(w.rows * 2 * 8));
  PSR_TRY(w.tau.ensure(nch * 8));
  PSR_TRY(w.kc.ensure(nch * 8));
  PSR_CUDA(cudaMemcpyAsync(w.tau.p, tau.data(), nch * 8, cudaMemcpyHostToDevice, st));
  PSR_CUDA(cudaMemcpyAsync(w.kc.p, kc.data(), nch * 8, cudaMemcpyHostToDevice, st));
  dim3 grid((unsigned)S, (unsigned)nch);
  const double *tp = w.tau.as<double>();
  float *cp = w.cube.as<float>();
  double *sp = w.chsum.as<double>();
  switch (o.kind) {
    case SAMPLE_U8:
      PSR_TRY(launch_cube_fold(grid, B, st, o.samples.as<uint8_t>(), o.ld, n, S, o.h.tsamp, nu,
                               nudot, tp, cp, sp));
      break;
    case SAMPLE_U16:
      PSR_TRY(launch_cube_fold(grid, B, st, o.samples.as<uint16_t>(), o.ld, n, S, o.h.tsamp, nu,
                               nudot, tp, cp, sp));
      break;
    default:
      PSR_TRY(launch_cube_fold(grid, B, st, o.samples.as<float>(), o.ld, n, S, o.h.tsamp, nu,
                               nudot, tp, cp, sp));
  }
  PSR_CUDA(cudaGetLastError());
  PSR_TRY(w.R.ensure(w.rows * (uint64_t)(B / 2) * sizeof(float2)));
  k_cube_dft<<<(unsigned)((w.rows + CB_ROWS - 1) / CB_ROWS), CB_NT, 0, st>>>(
      w.cube.as<float>(), w.rows, B, w.R.as<float2>());
  PSR_CUDA(cudaGetLastError());
  PSR_TRY(w.prof.ensure(16));
  k_cube_var<<<1, CB_NT, 0, st>>>(w.chsum.as<double>(), nch, S, n, w.prof.as<double>());
  PSR_CUDA(cudaGetLastError());
  double v = 0.0;
  PSR_CUDA(cudaMemcpyAsync(&v, w.prof.p, 8, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  w.var = v > 0.0 ? v : 1.0;
  return PSR_OK;
}

// J and gradient (in nu, nudot, DM) of every candidate.
int eval_cube(const DeviceObs &o, uint64_t n, int S, int B, double nu_r, double nudot_r,
              double dm_r, const std::vector<CandDev> &cand, CubeWork &w, std::vector<double> &J,
              std::vector<double> &grad, cudaStream_t st) {
  const int K = (int)cand.size();
  const int H = B / 2;
  const double Tsub = (double)n * o.h.tsamp / (double)S;
  PSR_TRY(w.cands.ensure(K * sizeof(CandDev)));
  PSR_TRY(w.prof.ensure((size_t)K * H * 2 * 8));
  PSR_TRY(w.g.ensure((size_t)K * H * sizeof(float2)));
  PSR_TRY(w.grad.ensure((size_t)K * 3 * 8));
  PSR_CUDA(cudaMemcpyAsync(w.cands.p, cand.data(), K * sizeof(CandDev), cudaMemcpyHostToDevice,
                           st));
  PSR_CUDA(cudaMemsetAsync(w.prof.p, 0, (size_t)K * H * 2 * 8, st));
  PSR_CUDA(cudaMemsetAsync(w.grad.p, 0, (size_t)K * 3 * 8, st));
  const int rows_per_cta = CB_NT;
  dim3 gp((unsigned)((w.rows + rows_per_cta - 1) / rows_per_cta), (unsigned)K);
  k_cube_harmonics<<<gp, CB_NT, 0, st>>>(w.R.as<float2>(), w.rows, S, B, w.kc.as<double>(), Tsub,
                                         nu_r, nudot_r, dm_r, w.cands.as<CandDev>(),
                                         rows_per_cta, w.prof.as<double>());
  PSR_CUDA(cudaGetLastError());
  std::vector<double> P((size_t)K * H * 2);
  PSR_CUDA(cudaMemcpyAsync(P.data(), w.prof.p, P.size() * 8, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  const double norm = (double)B * (double)n * w.var;
  std::vector<float2> A((size_t)K * H);
  J.assign(K, 0.0);
  for (int k = 0; k < K; ++k) {
    double j = 0.0;
    for (int h = 1; h <= H; ++h) {
      const double re = P[((size_t)k * H + h - 1) * 2], im = P[((size_t)k * H + h - 1) * 2 + 1];
      const double wk = h < H ? 2.0 : 1.0;
      j += wk * (re * re + im * im);
      A[(size_t)k * H + h - 1] = make_float2((float)(2.0 * wk * re / norm),
                                             (float)(-2.0 * wk * im / norm));
    }
    J[k] = j / norm;
  }
  PSR_CUDA(cudaMemcpyAsync(w.g.p, A.data(), A.size() * sizeof(float2), cudaMemcpyHostToDevice,
                           st));
  dim3 gg((unsigned)std::min<uint64_t>((w.rows + 255) / 256, 1024), (unsigned)K);
  k_cube_grad<<<gg, CB_NT, 0, st>>>(w.R.as<float2>(), w.rows, S, B, w.kc.as<double>(), Tsub,
                                    nu_r, nudot_r, dm_r, w.cands.as<CandDev>(),
                                    w.g.as<float2>(), w.grad.as<double>());
  PSR_CUDA(cudaGetLastError());
  grad.resize((size_t)K * 3);
  PSR_CUDA(cudaMemcpyAsync(grad.data(), w.grad.p, grad.size() * 8, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  return PSR_OK;
}

// Per-candidate quasi-Newton state (ascent on J in scaled coordinates).
struct Opt {
  double q[3] = {0, 0, 0}, g[3] = {0, 0, 0}, d[3] = {0, 0, 0}, qn[3] = {0, 0, 0};
  double H[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  double J = 0.0, slope = 0.0, alpha = 1.0, h0 = 1.0;
  int ls = 0;
  bool started = false, done = false;
  uint64_t evals = 0;
};

void set_direction(Opt &s) {
  for (int i = 0; i < 3; ++i)
    s.d[i] = s.H[i][0] * s.g[0] + s.H[i][1] * s.g[1] + s.H[i][2] * s.g[2];
  s.slope = s.d[0] * s.g[0] + s.d[1] * s.g[1] + s.d[2] * s.g[2];
  if (!(s.slope > 0.0)) {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) s.H[i][j] = i == j ? s.h0 : 0.0;
    for (int i = 0; i < 3; ++i) s.d[i] = s.h0 * s.g[i];
    s.slope = s.h0 * (s.g[0] * s.g[0] + s.g[1] * s.g[1] + s.g[2] * s.g[2]);
  }
  s.alpha = 1.0;
  s.ls = 0;
  if (!(s.slope > 0.0)) s.done = true;
}

}  // namespace

int cube_objective(const DeviceObs &o, uint64_t n, const psr_timing &ref, const psr_timing *theta,
                   uint64_t K, const RefineOptions &opt, double *Jout, double *gout,
                   cudaStream_t st) {
  const int B = (int)opt.bins, S = (int)opt.subints;
  if (B > CB_MAXB || B < 8 || S < 1 || K == 0) {
    set_error("cube_objective: 8..1024 bins, >= 1 subint and >= 1 point required");
    return PSR_EINVAL;
  }
  const double nu_r = 1.0 / ref.period_s, nudot_r = -ref.pdot * nu_r * nu_r;
  CubeWork w;
  PSR_TRY(build_cube(o, n, S, B, nu_r, nudot_r, ref.dm, w, st));
  std::vector<CandDev> cand(K);
  for (uint64_t k = 0; k < K; ++k) {
    cand[k].nu = 1.0 / theta[k].period_s;
    cand[k].nudot = -theta[k].pdot * cand[k].nu * cand[k].nu;
    cand[k].dm = theta[k].dm;
  }
  std::vector<double> J, grad;
  PSR_TRY(eval_cube(o, n, S, B, nu_r, nudot_r, ref.dm, cand, w, J, grad, st));
  for (uint64_t k = 0; k < K; ++k) {
    Jout[k] = J[k];
    if (gout) {
      gout[3 * k] = grad[3 * k];
      gout[3 * k + 1] = grad[3 * k + 1];
      gout[3 * k + 2] = grad[3 * k + 2];
    }
  }
  return PSR_OK;
}

int refine_cube_group(const DeviceObs &o, uint64_t n, const psr_timing *start, uint64_t K,
                      const RefineOptions &opt, psr_timing *out, double *Jout, uint64_t *evals,
                      CubeCache &cache, cudaStream_t st) {
  if (K == 0) return PSR_OK;
  const int B = (int)opt.bins, S = (int)opt.subints;
  if (B > CB_MAXB) {
    set_error("refine: at most 1024 bins");
    return PSR_EINVAL;
  }
  // Reference: the median start.
  std::vector<double> nus(K), dms(K);
  for (uint64_t k = 0; k < K; ++k) {
    nus[k] = 1.0 / start[k].period_s;
    dms[k] = start[k].dm;
  }
  std::vector<double> sn = nus, sd = dms;
  std::nth_element(sn.begin(), sn.begin() + K / 2, sn.end());
  std::nth_element(sd.begin(), sd.begin() + K / 2, sd.end());
  const double nu_r = sn[K / 2], dm_r = sd[K / 2];
  const double nudot_r = -start[K / 2].pdot * nu_r * nu_r;
  if (!cache.w) cache.w = new CubeWork();
  CubeWork &w = *cache.w;
  PSR_TRY(build_cube(o, n, S, B, nu_r, nudot_r, dm_r, w, st));
  const double T = (double)n * o.h.tsamp;
  double fmax = 0.0, fmin = 1e300;
  for (uint64_t c = 0; c < o.nch; ++c) {
    const double f = o.h.fch1 + (double)c * o.h.foff;
    fmax = std::fmax(fmax, f);
    fmin = std::fmin(fmin, f);
  }
  const double kspan = K_DM_C * (1.0 / (fmin * fmin) - 1.0 / (fmax * fmax));
  // Orthogonal scaled coordinates, as in the filterbank optimiser:
  // dnu = (2 q1 - 4 q2) / (B T), dnudot = 8 q2 / (B T^2), dDM = q3 s3.
  const double Bd = (double)B;
  const double s3 = kspan > 0.0 ? 1.0 / (nu_r * Bd * kspan) : 1.0;
  const double dm_hi = max_dm_for(o, n);
  std::vector<Opt> st8(K);
  auto theta = [&](uint64_t k, const double q[3]) {
    CandDev c;
    const double nu0 = 1.0 / start[k].period_s;
    const double nudot0 = -start[k].pdot * nu0 * nu0;
    c.nu = nu0 + (2.0 * q[0] - 4.0 * q[1]) / (Bd * T);
    c.nudot = nudot0 + 8.0 * q[1] / (Bd * T * T);
    double dm = start[k].dm + q[2] * s3;
    if (opt.dm_window > 0.0)
      dm = std::fmin(std::fmax(dm, start[k].dm - opt.dm_window), start[k].dm + opt.dm_window);
    c.dm = std::fmin(std::fmax(dm, 0.0), dm_hi);
    return c;
  };
  std::vector<double> J, grad;
  for (uint64_t round = 0; round < opt.max_evals; ++round) {
    std::vector<CandDev> batch;
    std::vector<uint64_t> who;
    for (uint64_t k = 0; k < K; ++k) {
      Opt &s = st8[k];
      if (s.done) continue;
      if (!s.started) {
        batch.push_back(theta(k, s.q));
      } else {
        for (int i = 0; i < 3; ++i) s.qn[i] = s.q[i] + s.alpha * s.d[i];
        batch.push_back(theta(k, s.qn));
      }
      who.push_back(k);
    }
    if (batch.empty()) break;
    PSR_TRY(eval_cube(o, n, S, B, nu_r, nudot_r, dm_r, batch, w, J, grad, st));
    for (size_t i = 0; i < who.size(); ++i) {
      Opt &s = st8[who[i]];
      ++s.evals;
      const double gq[3] = {grad[i * 3] * 2.0 / (Bd * T),
                            grad[i * 3] * (-4.0 / (Bd * T)) + grad[i * 3 + 1] * 8.0 / (Bd * T * T),
                            grad[i * 3 + 2] * s3};
      if (!s.started) {
        s.started = true;
        s.J = J[i];
        for (int j = 0; j < 3; ++j) s.g[j] = gq[j];
        const double gn = std::sqrt(gq[0] * gq[0] + gq[1] * gq[1] + gq[2] * gq[2]);
        s.h0 = gn > 0.0 ? 1.0 / gn : 1.0;
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b) s.H[a][b] = a == b ? s.h0 : 0.0;
        set_direction(s);
        continue;
      }
      if (J[i] >= s.J + 1e-4 * s.alpha * s.slope) {
        double sv[3], yv[3], maxstep = 0.0;
        for (int j = 0; j < 3; ++j) {
          sv[j] = s.qn[j] - s.q[j];
          yv[j] = -(gq[j] - s.g[j]);
          maxstep = std::fmax(maxstep, std::fabs(sv[j]));
        }
        const double sy = sv[0] * yv[0] + sv[1] * yv[1] + sv[2] * yv[2];
        if (sy > 1e-12) {
          double Hy[3], yHy = 0.0;
          for (int a = 0; a < 3; ++a)
            Hy[a] = s.H[a][0] * yv[0] + s.H[a][1] * yv[1] + s.H[a][2] * yv[2];
          for (int a = 0; a < 3; ++a) yHy += yv[a] * Hy[a];
          for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
              s.H[a][b] += (sy + yHy) * sv[a] * sv[b] / (sy * sy) -
                           (Hy[a] * sv[b] + sv[a] * Hy[b]) / sy;
        }
        for (int j = 0; j < 3; ++j) {
          s.q[j] = s.qn[j];
          s.g[j] = gq[j];
        }
        s.J = J[i];
        if (maxstep < opt.tol) s.done = true;
        else set_direction(s);
      } else {
        s.alpha *= 0.5;
        if (++s.ls >= 12) s.done = true;
      }
    }
  }
  for (uint64_t k = 0; k < K; ++k) {
    const CandDev c = theta(k, st8[k].q);
    out[k].period_s = 1.0 / c.nu;
    out[k].pdot = -c.nudot / (c.nu * c.nu);
    out[k].dm = c.dm;
    if (Jout) Jout[k] = st8[k].J;
    if (evals) evals[k] = st8[k].evals;
  }
  return PSR_OK;
}

}  // namespace psr
