// K5 power normalisation + birdies, K6 harmonic sums + peaks, K7 per-trial
// sort/dedupe (search/src/lib.rs:45-144).
//
// Normalisation: every 64-bin block b is divided by
//   scale_b = max(max(median(raw[lo..hi]) / ln2, floor), 1e-20),
//   lo = max(64b-128, 1), hi = min(64b+192, len), floor = 1e-6 * mean(raw).
// The median is exact: each 64-bin chunk is sorted once per CTA (a register
// bitonic network per thread; non-negative floats order like their bit
// patterns), elements
// provably below the window's rank-(cnt/2) element are skipped with binary
// searches, and a 5-way merge walk over the sorted chunks finds it.  Normalised power is never
// stored: pw(i) = raw[i] / scale[i>>6], zero for i == 0 and birdie bins.
//
// Harmonic sums follow the reference's f64 arithmetic exactly.  The f64 work
// is only done where it can matter: h = 1 scores are pw(k) or pw(k+1) minus 1,
// so a bin whose larger neighbour cannot reach the threshold is skipped
// before the parabolic offset is computed; h >= 2 scores exist only where
// pw(k) >= 4 (search/src/lib.rs:85-87).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "psr_internal.h"

namespace psr {
namespace {

constexpr int SC_NT = 256;               // threads per CTA, one chunk sort each
constexpr int SC_CH = SC_NT;             // chunks staged per CTA
constexpr int SC_G = SC_CH - 4;          // blocks per CTA (chunks b-2 .. b+2 each)
constexpr float LN2F = 0.693147180559945309f;

__device__ __forceinline__ uint32_t fbits(float f) { return __float_as_uint(f); }

// Number of elements <= key in a sorted chunk of 64 keys (invalid slots hold
// 0xffffffff, above every finite float pattern).  Branchless, 7 probes.
__device__ __forceinline__ int count_le64(const uint32_t *a, uint32_t key) {
  int pos = (a[31] <= key) ? 32 : 0;
  pos += (a[pos + 15] <= key) ? 16 : 0;
  pos += (a[pos + 7] <= key) ? 8 : 0;
  pos += (a[pos + 3] <= key) ? 4 : 0;
  pos += (a[pos + 1] <= key) ? 2 : 0;
  pos += (a[pos] <= key) ? 1 : 0;
  pos += (a[pos] <= key) ? 1 : 0;
  return pos;
}

// Chunks are stored with a 65-word stride so that threads probing the same
// index of different chunks hit different banks.
constexpr int SC_STRIDE = 65;

struct RawCand {
  double score;
  double freq;
  uint32_t k;
  uint32_t h;
};

struct HarmArgs {
  const float *power;
  uint64_t ldp;
  uint64_t plen;
  const float *scale;
  uint64_t lds;
  const double *birdies;
  int nbirdies;
  double bin_hz;
  double threshold;
  float t1;  // smallest float v with (double)v - 1.0 >= threshold
  uint64_t first;
  uint64_t end[6];  // end_h for h = 1,2,4,8,16,32 (0 when the h loop is skipped)
  RawCand *raw;
  unsigned *raw_count;
  uint64_t raw_cap;
  unsigned *overflow;
};

__device__ __forceinline__ float pw(const HarmArgs &a, const float *raw, const float *sc,
                                    uint64_t i) {
  if (i == 0) return 0.0f;
  float v = __fdiv_rn(raw[i], sc[i >> 6]);
  if (a.nbirdies) {
    const double f = (double)i * a.bin_hz;
    for (int q = 0; q < a.nbirdies; ++q)
      if (fabs(__dsub_rn(f, a.birdies[2 * q])) <= a.birdies[2 * q + 1]) return 0.0f;
  }
  return v;
}

// Parabolic offset (search/src/lib.rs:91-96).
__device__ __forceinline__ double offset_at(const float *raw, uint64_t k) {
  const double a = (double)raw[k - 1], b = (double)raw[k], c = (double)raw[k + 1];
  const double curv = __dadd_rn(__dsub_rn(a, __dmul_rn(2.0, b)), c);
  if (curv < 0.0) {
    const double o = __ddiv_rn(__dmul_rn(0.5, __dsub_rn(a, c)), curv);
    return fmin(fmax(o, -0.5), 0.5);
  }
  return 0.0;
}

__device__ __forceinline__ double inv_sqrt_div(double x, int hi) {
  // (sum - h) / sqrt(h): sqrt(h) correctly rounded as in Rust's f64::sqrt.
  switch (hi) {
    case 0: return x;
    case 1: return __ddiv_rn(x, 1.4142135623730951);
    case 2: return __dmul_rn(x, 0.5);
    case 3: return __ddiv_rn(x, 2.8284271247461903);
    case 4: return __dmul_rn(x, 0.25);
    default: return __ddiv_rn(x, 5.656854249492381);
  }
}

// Whether (sum - h) / sqrt(h) can reach thr, without the f64 division where
// it clearly cannot: x * RN(1/sqrt(h)) is within 2^-50 (relative) of the
// correctly rounded quotient, so below thr by more than |thr| 2^-49 it is
// below for certain.  Levels with h = 1, 4, 16 scale exactly: always true.
__device__ __forceinline__ bool may_reach(double x, int hi, double thr) {
  if ((hi & 1) == 0) return true;
  constexpr double r1 = 0.7071067811865476;  // RN(1/sqrt(2)); / 2 and / 4 are exact
  const double r = hi == 1 ? r1 : hi == 3 ? r1 * 0.5 : r1 * 0.25;
  return __dmul_rn(x, r) >= thr - fabs(thr) * 0x1p-49;
}

// Full score of harmonic level hi (h = 1 << hi) at bin k (k in [first, end]).
__device__ double score_at(const HarmArgs &a, const float *raw, const float *sc, uint64_t k,
                           int hi) {
  const int h = 1 << hi;
  if (h > 1 && pw(a, raw, sc, k) < 4.0f) return -INFINITY;
  const double off = offset_at(raw, k);
  const double kf = __dadd_rn((double)k, off);
  double sum = -0.0;
  for (int j = 1; j <= h; ++j) {
    const double pos = __dmul_rn(kf, (double)j);
    uint64_t idx = (uint64_t)round(pos);
    if (idx > a.plen - 1) idx = a.plen - 1;
    sum = __dadd_rn(sum, (double)pw(a, raw, sc, idx));
  }
  return inv_sqrt_div(__dsub_rn(sum, (double)h), hi);
}

// Appends a raw candidate.  The lanes of a warp that emit together (all for
// the CTA's one trial) take consecutive slots: a ballot of the converged
// lanes, one atomic by the lowest, the base broadcast by a shuffle and each
// lane's rank among them.  The order of the raw list does not matter:
// k_select orders it by (score, h, k).
__device__ void emit(const HarmArgs &a, uint64_t trial, const float *raw, uint64_t k, int hi,
                     double score) {
  const unsigned mask = __activemask();
  const int lane = (int)(threadIdx.x & 31);
  const int leader = __ffs(mask) - 1;
  unsigned base = 0;
  if (lane == leader) base = atomicAdd(&a.raw_count[trial], (unsigned)__popc(mask));
  base = __shfl_sync(mask, base, leader);
  const unsigned slot = base + (unsigned)__popc(mask & ((1u << lane) - 1u));
  if (slot >= a.raw_cap) {
    atomicOr(a.overflow, 1u);
    return;
  }
  const double off = offset_at(raw, k);
  RawCand c;
  c.score = score;
  c.freq = __dmul_rn(__dadd_rn((double)k, off), a.bin_hz);
  c.k = (uint32_t)k;
  c.h = (uint32_t)hi;
  a.raw[trial * a.raw_cap + slot] = c;
}


// round(RN(kf * j)) for a positive normal double kf and 1 <= j <= 32, in
// exact 64-bit integer arithmetic: kf = m * 2^E (53-bit m), the product m*j
// is exact in 58 bits, rounded to 53 bits (nearest, ties to even) as the FPU
// would, then rounded to an integer half away from zero as f64::round does.
// Bit-identical to (uint64_t)round(__dmul_rn(kf, (double)j)).
__device__ __forceinline__ uint64_t round_mul(double kf, uint32_t j) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(kf);
  const int E = (int)((bits >> 52) & 0x7ff) - 1075;
  const unsigned long long m = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  unsigned long long q = m * (unsigned long long)j;
  int F = E;
  const int nb = 64 - __clzll((long long)q);
  if (nb > 53) {
    const int sh = nb - 53;
    const unsigned long long rem = q & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
    q >>= sh;
    F += sh;
    if (rem > half || (rem == half && (q & 1ull))) ++q;
    if (q >> 53) {
      q >>= 1;
      ++F;
    }
  }
  if (F >= 0) return q << F;
  const int s = -F;
  if (s >= 64) return 0;
  const unsigned long long ip = q >> s, fr = q & ((1ull << s) - 1ull);
  return ip + (fr >= (1ull << (s - 1)) ? 1ull : 0ull);
}

// All harmonic levels h >= 2 of one gated bin (pw(k) >= 4), one lane per
// bin: the offset is computed once, the harmonic positions and gathers are
// issued together, and the f64 sums accumulate in j order (the reference's
// per-h sums are the same prefix sums).  NL = number of levels (5: h <= 16,
// 6: h <= 32).
template <int NL>
__device__ void harm_item(const HarmArgs &a, uint64_t trial, const float *raw, const float *sc,
                          uint64_t k) {
  constexpr int HMAX = 1 << (NL - 1);
  int hmax = 0;
#pragma unroll
  for (int hi = 1; hi < NL; ++hi)
    if (a.end[hi] != 0 && k + 1 <= a.end[hi]) hmax = hi;
  if (hmax == 0 || pw(a, raw, sc, k) < 4.0f) return;  // queue entries are a superset
  const double kf = __dadd_rn((double)k, offset_at(raw, k));
  const int H = 1 << hmax;
  float v[HMAX];
#pragma unroll
  for (int j = 1; j <= HMAX; ++j) {
    float x = 0.0f;
    if (j <= H) {
      uint64_t idx = round_mul(kf, (uint32_t)j);
      if (idx > a.plen - 1) idx = a.plen - 1;
      x = pw(a, raw, sc, idx);
    }
    v[j - 1] = x;
  }
  double sum = -0.0;
#pragma unroll
  for (int hi = 1; hi < NL; ++hi) {
    if (hi > hmax) break;
    const int h = 1 << hi;
    // harmonics j = h/2+1 .. h (v[j-1]); for h = 2 also j = 1
#pragma unroll
    for (int j = (hi == 1 ? 0 : h / 2); j < h; ++j) sum = __dadd_rn(sum, (double)v[j]);
    const double xs = __dsub_rn(sum, (double)h);
    if (!may_reach(xs, hi, a.threshold)) continue;
    const double s = inv_sqrt_div(xs, hi);
    if (s >= a.threshold) {
      const double sm = score_at(a, raw, sc, k - 1, hi);
      const double sp = score_at(a, raw, sc, k + 1, hi);
      if (s > sm && s >= sp) emit(a, trial, raw, k, hi, s);
    }
  }
}

// Gate queues: per trial the bins that pass the h = 1 gate (q1) and the
// h >= 2 gate (q2); capacity qcap each, counts n1/n2.
struct GateArgs {
  uint32_t *q1, *q2;
  unsigned *n1, *n2;
  uint64_t qcap;
};

constexpr int SCG_OWN = SC_G * 64;  // bins of the CTA's own blocks
constexpr int SCG_LQ = 1024;        // local queue slots (overflow goes to global)
constexpr size_t SCG_SMEM = (size_t)SC_CH * SC_STRIDE * 4 + (size_t)(SC_G + 4) * 4 +
                            (size_t)SCG_LQ * 2 * 2;

// Normalisation scales of 124 blocks per CTA, then the harmonic gates on the
// CTA's own bins while they are hot in L2.  An h = 1 peak needs
// max(pw(k), pw(k+1)) >= t1 (t1 = the smallest float whose f64 value minus 1
// reaches the threshold; score_1(k) is pw(k) - 1 or pw(k+1) - 1), and h >= 2
// scores exist only where pw(k) >= 4.  The gates are conservative supersets:
// pw is estimated as raw * (1/scale) and a bin is queued unless the estimate
// is below the threshold by more than 4e-7 relative (the estimate is within
// 2e-7 of the correctly rounded quotient); birdies are ignored and the last
// bin, whose neighbour's scale belongs to the next CTA, is always queued.
// The item kernel evaluates every queued bin exactly.
__global__ void __launch_bounds__(SC_NT)
    k_scales_gate(HarmArgs a, const double *__restrict__ psum, uint32_t npsum,
                  uint64_t nblocks, float *__restrict__ scale_out, GateArgs g) {
  extern __shared__ __align__(16) uint32_t dsm[];
  uint32_t *ch = dsm;                                // SC_CH x SC_STRIDE (sorted chunks)
  float *inv_s = reinterpret_cast<float *>(ch + SC_CH * SC_STRIDE);  // 1/scale per block
  uint16_t *lq1 = reinterpret_cast<uint16_t *>(inv_s + SC_G + 4);
  uint16_t *lq2 = lq1 + SCG_LQ;
  __shared__ float floor_s;
  __shared__ int c1, c2;
  __shared__ unsigned base1, base2;
  const uint64_t plen = a.plen;
  const uint64_t trial = blockIdx.y;
  const float *raw = a.power + trial * a.ldp;
  const long long b0 = (long long)blockIdx.x * SC_G;
  const long long c_first = b0 - 2;  // chunk index of local chunk 0
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) {  // floor: mean of the raw power from the FFT's partial sums
    double s = 0.0;
    for (uint32_t i = lane; i < npsum; i += 32) s += psum[trial * npsum + i];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) floor_s = (float)(s / (double)plen * 1e-6);
  }
  if (threadIdx.x == 0) c1 = c2 = 0;
  // Stage the bins of all chunks (16-byte loads, four in flight per thread);
  // out-of-range chunks and bin 0 hold the sentinel 0xffffffff.
  constexpr int NV = SC_CH * 64;
  constexpr int NV4 = NV / 4;
  static_assert(NV4 % (4 * SC_NT) == 0, "staging loop covers the chunks exactly");
  const long long e_first = c_first * 64;  // a multiple of 4: 16-byte aligned loads
  for (int base = 0; base < NV4; base += 4 * SC_NT) {
    uint4 v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const long long e = e_first + 4ll * (base + u * SC_NT + (int)threadIdx.x);
      if (e >= 1 && e + 3 < (long long)plen) {
        v[u] = *reinterpret_cast<const uint4 *>(raw + e);
      } else {
        uint32_t t[4];
#pragma unroll
        for (int j = 0; j < 4; ++j)
          t[j] = (e + j >= 1 && e + j < (long long)plen) ? fbits(raw[e + j]) : 0xffffffffu;
        v[u] = make_uint4(t[0], t[1], t[2], t[3]);
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = 4 * (base + u * SC_NT + (int)threadIdx.x);
      uint32_t *dst = ch + (i >> 6) * SC_STRIDE + (i & 63);  // one chunk row
      dst[0] = v[u].x;
      dst[1] = v[u].y;
      dst[2] = v[u].z;
      dst[3] = v[u].w;
    }
  }
  __syncthreads();
  {
    // Thread t sorts chunk t in registers: Batcher's odd-even merge sort
    // network (543 compare-exchanges for 64 keys), fully unrolled, so every
    // register index is static and there are no shuffles.  The stride-65
    // layout makes these row reads bank-conflict free.
    uint32_t x[64];
    uint32_t *row = ch + threadIdx.x * SC_STRIDE;
#pragma unroll
    for (int i = 0; i < 64; ++i) x[i] = row[i];
    // (merge step (p, k) compares a with a + k for every a >= k % p with
    // (a - k % p) mod 2k < k, both in one block of 2p)
#pragma unroll
    for (int p = 1; p < 64; p <<= 1)
#pragma unroll
      for (int k = p; k >= 1; k >>= 1)
#pragma unroll
        for (int a = 0; a < 64; ++a) {
          const int c = a + k, j0 = k % p;
          if (c < 64 && a >= j0 && (a - j0) % (2 * k) < k && a / (2 * p) == c / (2 * p)) {
            const uint32_t p0 = x[a], p1 = x[c];
            x[a] = min(p0, p1);
            x[c] = max(p0, p1);
          }
        }
#pragma unroll
    for (int i = 0; i < 64; ++i) row[i] = x[i];
  }
  __syncthreads();
  const long long b = b0 + threadIdx.x;
  if (threadIdx.x < SC_G && b < (long long)nblocks) {
    const long long center = b * 64;
    const long long lo = max(center - 128, 1ll);
    const long long hi = min(center + 192, (long long)plen);
    const int r = (int)(hi - lo) / 2;
    // The window is local chunks threadIdx.x .. threadIdx.x + 4 (chunks
    // b-2..b+2), each sorted and padded with sentinels above every value.
    const uint32_t *w = ch + threadIdx.x * SC_STRIDE;
    // Rank-bound skips: with p_d elements of chunk d already known to lie
    // below the target and rr = r - sum(p_d), let y = min_d A_d[p_d + rr/5].
    // Each chunk has at most rr/5 unskipped elements below y, so at most rr
    // elements below y remain and the rank-r element is >= y: skip them.
    // Every round shrinks rr geometrically; a short merge walk finishes.
    int p[5] = {0, 0, 0, 0, 0};
    int rr = r;
    for (int round = 0; round < 6; ++round) {
      const int q = rr / 5;
      if (q == 0) break;
      uint32_t y = 0xffffffffu;
#pragma unroll
      for (int d = 0; d < 5; ++d)
        if (p[d] + q < 64) y = min(y, w[d * SC_STRIDE + p[d] + q]);
      if (y == 0u) break;
      int adv = 0;
#pragma unroll
      for (int d = 0; d < 5; ++d) {
        const int np = count_le64(w + d * SC_STRIDE, y - 1u);  // elements < y
        adv += np - p[d];
        p[d] = np;
      }
      rr -= adv;
      if (adv == 0) break;
    }
    // 5-way merge walk over the rest: advance the smallest head rr times; the
    // smallest head is then the rank-r element.
    uint32_t hd[5];
#pragma unroll
    for (int d = 0; d < 5; ++d) hd[d] = p[d] < 64 ? w[d * SC_STRIDE + p[d]] : 0xffffffffu;
    for (int step = 0; step < rr; ++step) {
      uint32_t m = hd[0];
      int am = 0;
#pragma unroll
      for (int d = 1; d < 5; ++d)
        if (hd[d] < m) {
          m = hd[d];
          am = d;
        }
#pragma unroll
      for (int d = 0; d < 5; ++d)
        if (d == am) {
          ++p[d];
          hd[d] = p[d] < 64 ? w[d * SC_STRIDE + p[d]] : 0xffffffffu;
        }
    }
    uint32_t med_k = hd[0];
#pragma unroll
    for (int d = 1; d < 5; ++d) med_k = min(med_k, hd[d]);
    const float sc = fmaxf(fmaxf(__fdiv_rn(__uint_as_float(med_k), LN2F), floor_s), 1e-20f);
    inv_s[threadIdx.x] = __frcp_rn(sc);
    scale_out[trial * a.lds + b] = sc;
  }
  __syncthreads();
  // Gates on the CTA's own bins (raw values re-read; they are hot in L2).
  const uint64_t kb0 = (uint64_t)b0 * 64;
  const float t1lo = a.t1 > 0.0f ? a.t1 * (1.0f - 4e-7f) : -INFINITY;
  const float t4lo = 4.0f * (1.0f - 4e-7f);
  const float tmin = fminf(t1lo, t4lo);
  uint32_t *gq1 = g.q1 + trial * g.qcap, *gq2 = g.q2 + trial * g.qcap;
  // Four consecutive bins per thread (one 16-byte load, one block scale);
  // the fourth bin's neighbour is the next group's first.
  for (int i4 = threadIdx.x; i4 < SCG_OWN / 4; i4 += SC_NT) {
    const int i = 4 * i4;
    const uint64_t k = kb0 + (uint64_t)i;
    if (k + 3 < a.first + 1 || k + 1 > a.end[0]) continue;  // no bin in [first+1, end_1 - 1]
    const float4 r4 = *reinterpret_cast<const float4 *>(raw + k);
    const float inv = inv_s[i >> 6];
    const float e[4] = {r4.x * inv, r4.y * inv, r4.z * inv, r4.w * inv};
    const float nx =
        (i + 4 < SCG_OWN && k + 4 <= a.end[0]) ? raw[k + 4] * inv_s[(i + 4) >> 6] : 0.0f;
    // Most groups pass neither gate: every estimate (and the neighbour's)
    // below both thresholds queues nothing (the CTA's last group excepted).
    if (i + 4 < SCG_OWN &&
        fmaxf(fmaxf(fmaxf(e[0], e[1]), fmaxf(e[2], e[3])), nx) < tmin)
      continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint64_t kj = k + (uint64_t)j;
      if (kj < a.first + 1 || kj + 1 > a.end[0]) continue;
      const float e0 = e[j];
      bool pass1 = true;
      if (i + j + 1 < SCG_OWN) pass1 = fmaxf(e0, j < 3 ? e[j + 1] : nx) >= t1lo;
      if (pass1) {
        const int slot = atomicAdd(&c1, 1);
        if (slot < SCG_LQ) {
          lq1[slot] = (uint16_t)(i + j);
        } else {
          const unsigned gi = atomicAdd(&g.n1[trial], 1u);
          if (gi < g.qcap) gq1[gi] = (uint32_t)kj;
          else atomicOr(a.overflow, 1u);
        }
      }
      if (e0 >= t4lo) {
        const int slot = atomicAdd(&c2, 1);
        if (slot < SCG_LQ) {
          lq2[slot] = (uint16_t)(i + j);
        } else {
          const unsigned gi = atomicAdd(&g.n2[trial], 1u);
          if (gi < g.qcap) gq2[gi] = (uint32_t)kj;
          else atomicOr(a.overflow, 1u);
        }
      }
    }
  }
  __syncthreads();
  const int m1 = min(c1, SCG_LQ), m2 = min(c2, SCG_LQ);
  if (threadIdx.x == 0) {
    base1 = atomicAdd(&g.n1[trial], (unsigned)m1);
    base2 = atomicAdd(&g.n2[trial], (unsigned)m2);
  }
  __syncthreads();
  if (threadIdx.x == 0 && (base1 + m1 > g.qcap || base2 + m2 > g.qcap)) atomicOr(a.overflow, 1u);
  for (int i = threadIdx.x; i < m1 && base1 + i < g.qcap; i += SC_NT)
    gq1[base1 + i] = (uint32_t)(kb0 + lq1[i]);
  for (int i = threadIdx.x; i < m2 && base2 + i < g.qcap; i += SC_NT)
    gq2[base2 + i] = (uint32_t)(kb0 + lq2[i]);
}

// Exact evaluation of the gated bins, one bin per thread: h = 1 peaks for
// q1 entries, all harmonic levels h >= 2 for q2 entries.
constexpr int HI_NT = 256;
constexpr int HI_CTAS_PER_TRIAL = 12;

template <int NL>
__global__ void __launch_bounds__(HI_NT) k_harm_items(HarmArgs a, GateArgs g) {
  const uint64_t trial = blockIdx.y;
  const float *raw = a.power + trial * a.ldp;
  const float *sc = a.scale + trial * a.lds;
  const unsigned n1 = min(g.n1[trial], (unsigned)g.qcap), n2 = min(g.n2[trial], (unsigned)g.qcap);
  const uint32_t *q1 = g.q1 + trial * g.qcap, *q2 = g.q2 + trial * g.qcap;
  for (unsigned idx = blockIdx.x * HI_NT + threadIdx.x; idx < n1 + n2;
       idx += gridDim.x * HI_NT) {
    if (idx < n1) {
      const uint64_t k = q1[idx];
      const double s = score_at(a, raw, sc, k, 0);
      if (s >= a.threshold) {
        const double sm = score_at(a, raw, sc, k - 1, 0);
        const double sp = score_at(a, raw, sc, k + 1, 0);
        if (s > sm && s >= sp) emit(a, trial, raw, k, 0, s);
      }
    } else {
      harm_item<NL>(a, trial, raw, sc, q2[idx - n1]);
    }
  }
}

// Orderable key: score descending, then (h, k) ascending = the reference's
// insertion order under its stable sort (search/src/lib.rs:130).
__device__ __forceinline__ unsigned long long score_key_desc(double s) {
  unsigned long long b = (unsigned long long)__double_as_longlong(s);
  unsigned long long asc = (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
  return ~asc;
}

constexpr int SEL_CAP = 2048;
constexpr int SEL_NT = 1024;

struct SelArgs {
  const RawCand *raw;
  const unsigned *raw_count;
  uint64_t raw_cap;
  const double *trial_dm;
  double tol;  // 1 / (len * tsamp)
  uint64_t max_candidates;
  psr_candidate *kept;
  unsigned *kept_count;
};

__device__ __forceinline__ bool key_less(unsigned long long ka, uint32_t sa,
                                         unsigned long long kb, uint32_t sb) {
  return ka < kb || (ka == kb && sa < sb);
}

__global__ void __launch_bounds__(SEL_NT) k_select(SelArgs a) {
  __shared__ unsigned long long key[SEL_CAP];
  __shared__ uint32_t seq[SEL_CAP];
  __shared__ uint32_t idx[SEL_CAP];
  __shared__ double kept_f[64];
  __shared__ int nk;
  const uint64_t trial = blockIdx.x;
  const RawCand *rc = a.raw + trial * a.raw_cap;
  const unsigned n = min(a.raw_count[trial], (unsigned)a.raw_cap);
  psr_candidate *out = a.kept + trial * a.max_candidates;
  const double dm = a.trial_dm[trial];
  if (threadIdx.x == 0) nk = 0;
  if (n <= SEL_CAP) {
    unsigned P = 1;
    while (P < n) P <<= 1;
    for (unsigned i = threadIdx.x; i < P; i += blockDim.x) {
      if (i < n) {
        key[i] = score_key_desc(rc[i].score);
        seq[i] = (rc[i].h << 24) | rc[i].k;
        idx[i] = i;
      } else {
        key[i] = ~0ull;
        seq[i] = 0xffffffffu;
        idx[i] = 0xffffffffu;
      }
    }
    __syncthreads();
    for (unsigned k = 2; k <= P; k <<= 1)
      for (unsigned j = k >> 1; j > 0; j >>= 1) {
        for (unsigned i = threadIdx.x; i < P; i += blockDim.x) {
          const unsigned l = i ^ j;
          if (l > i) {
            const bool up = (i & k) == 0;
            const bool gt = key_less(key[l], seq[l], key[i], seq[i]);
            if (gt == up) {
              unsigned long long tk = key[i];
              key[i] = key[l];
              key[l] = tk;
              uint32_t ts = seq[i];
              seq[i] = seq[l];
              seq[l] = ts;
              uint32_t ti = idx[i];
              idx[i] = idx[l];
              idx[l] = ti;
            }
          }
        }
        __syncthreads();
      }
    // Sequential dedupe by warp 0 (search/src/lib.rs:131-143).
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
      int kc = 0;
      for (unsigned i = 0; i < n && (uint64_t)kc < a.max_candidates; ++i) {
        const RawCand c = rc[idx[i]];
        bool dup = false;
        for (int q = lane; q < kc; q += 32) dup |= fabs(__dsub_rn(kept_f[q], c.freq)) < a.tol;
        dup = __any_sync(0xffffffffu, dup);
        if (!dup) {
          if (lane == 0) {
            kept_f[kc] = c.freq;
            psr_candidate o;
            o.frequency_hz = c.freq;
            o.period_s = __ddiv_rn(1.0, c.freq);
            o.dm = dm;
            o.harmonics = 1ull << c.h;
            o.score = c.score;
            out[kc] = o;
          }
          ++kc;
          __syncwarp();
        }
      }
      if (lane == 0) a.kept_count[trial] = (unsigned)kc;
    }
    return;
  }
  // More raw candidates than fit in shared memory: repeated arg-max over the
  // unsorted list (exact order; only reached by pathological spectra).
  __shared__ unsigned long long best_k[SEL_NT / 32];
  __shared__ uint32_t best_s[SEL_NT / 32], best_i[SEL_NT / 32];
  __shared__ unsigned long long last_k;
  __shared__ uint32_t last_s;
  if (threadIdx.x == 0) {
    last_k = 0;
    last_s = 0;
  }
  __syncthreads();
  bool started = false;
  for (;;) {
    unsigned long long bk = ~0ull;
    uint32_t bs = 0xffffffffu, bi = 0xffffffffu;
    for (unsigned i = threadIdx.x; i < n; i += blockDim.x) {
      const unsigned long long kk = score_key_desc(rc[i].score);
      const uint32_t ss = (rc[i].h << 24) | rc[i].k;
      if (started && !key_less(last_k, last_s, kk, ss)) continue;  // already consumed
      if (key_less(kk, ss, bk, bs)) {
        bk = kk;
        bs = ss;
        bi = i;
      }
    }
    for (int o = 16; o; o >>= 1) {
      unsigned long long ok = __shfl_xor_sync(0xffffffffu, bk, o);
      uint32_t os = __shfl_xor_sync(0xffffffffu, bs, o);
      uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (key_less(ok, os, bk, bs)) {
        bk = ok;
        bs = os;
        bi = oi;
      }
    }
    if ((threadIdx.x & 31) == 0) {
      best_k[threadIdx.x >> 5] = bk;
      best_s[threadIdx.x >> 5] = bs;
      best_i[threadIdx.x >> 5] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long k0 = ~0ull;
      uint32_t s0 = 0xffffffffu, i0 = 0xffffffffu;
      for (int w = 0; w < SEL_NT / 32; ++w)
        if (key_less(best_k[w], best_s[w], k0, s0)) {
          k0 = best_k[w];
          s0 = best_s[w];
          i0 = best_i[w];
        }
      best_i[0] = i0;
      if (i0 != 0xffffffffu) {
        last_k = k0;
        last_s = s0;
        const RawCand c = rc[i0];
        bool dup = false;
        for (int q = 0; q < nk; ++q) dup |= fabs(__dsub_rn(kept_f[q], c.freq)) < a.tol;
        if (!dup) {
          kept_f[nk] = c.freq;
          psr_candidate o;
          o.frequency_hz = c.freq;
          o.period_s = __ddiv_rn(1.0, c.freq);
          o.dm = dm;
          o.harmonics = 1ull << c.h;
          o.score = c.score;
          out[nk] = o;
          ++nk;
        }
      }
    }
    __syncthreads();
    started = true;
    if (best_i[0] == 0xffffffffu || (uint64_t)nk >= a.max_candidates) break;
    __syncthreads();
  }
  if (threadIdx.x == 0) a.kept_count[trial] = (unsigned)nk;
}

}  // namespace

// Buffers for up to `outer` trials of raw candidates and `inner` trials of
// normalisation scales; uploads the birdie list.
int spectrum_prepare(const FftPlan &p, const SpecConfig &c, uint64_t outer, uint64_t inner,
                     SpecWork &w, cudaStream_t st) {
  if (c.max_candidates > 64 || c.max_candidates < 1) {
    set_error("search: 1..64 candidates per trial are supported");
    return PSR_EINVAL;
  }
  const uint64_t plen = p.M + 1;
  const uint64_t nblocks = (plen + 63) / 64;
  w.lds = ((nblocks + 63) / 64) * 64;
  if (w.raw_cap == 0) w.raw_cap = 2048;
  PSR_TRY(w.scale.ensure(outer * w.lds * 4));
  (void)inner;
  PSR_TRY(w.raw.ensure(outer * w.raw_cap * sizeof(RawCand)));
  PSR_TRY(w.raw_count.ensure(outer * 4));
  PSR_TRY(w.overflow.ensure(16));
  // Gated bins are ~2% of a noise spectrum; a quarter of the bins is ample
  // and an overflow (flagged) reruns the chunk with room for every bin.
  w.qcap = w.queue_full ? plen : plen / 4 + 1024;
  PSR_TRY(w.gq.ensure(2 * outer * w.qcap * 4));
  PSR_TRY(w.gn.ensure(2 * outer * 4 + 16));
  PSR_TRY(w.birdies.ensure(std::max<size_t>(c.birdies.size(), 2) * 8));
  if (!c.birdies.empty())
    PSR_CUDA(cudaMemcpyAsync(w.birdies.p, c.birdies.data(), c.birdies.size() * 8,
                             cudaMemcpyHostToDevice, st));
  return PSR_OK;
}

int spectrum_reset(SpecWork &w, uint64_t outer_trials, cudaStream_t st) {
  PSR_CUDA(cudaMemsetAsync(w.raw_count.p, 0, outer_trials * 4, st));
  PSR_CUDA(cudaMemsetAsync(w.overflow.p, 0, 16, st));
  PSR_CUDA(cudaMemsetAsync(w.gn.p, 0, 2 * outer_trials * 4, st));
  w.outer_trials = outer_trials;
  return PSR_OK;
}

// Normalisation scales and harmonic peaks of `ntrials` spectra; their raw
// candidates go to slots [slot0, slot0 + ntrials) of the outer chunk.
namespace {
HarmArgs harm_args(const FftPlan &p, const SpecConfig &c, const float *d_power, uint64_t ldp,
                   SpecWork &w) {
  const uint64_t plen = p.M + 1;
  // search/src/lib.rs:62, 73-78
  const double bin_hz = 1.0 / ((double)p.N * c.tsamp);
  HarmArgs a{};
  a.power = d_power;
  a.ldp = ldp;
  a.plen = plen;
  a.scale = w.scale.as<float>();
  a.lds = w.lds;
  a.birdies = w.birdies.as<double>();
  a.nbirdies = (int)(c.birdies.size() / 2);
  a.bin_hz = bin_hz;
  a.threshold = c.threshold;
  const double firstf = std::fmax(std::ceil(c.min_hz / bin_hz), 1.0);
  const uint64_t first = (uint64_t)firstf;
  const double lastf = std::floor(std::fmin(c.max_hz, 0.5 / c.tsamp) / bin_hz);
  const uint64_t last = std::min<uint64_t>(lastf <= 0.0 ? 0 : (uint64_t)lastf, plen - 2);
  a.first = first;
  for (int hi = 0; hi < c.levels; ++hi) {
    const uint64_t h = 1ull << hi;
    const uint64_t e = std::min(last, (plen - 2) / h);
    a.end[hi] = (e <= first + 1) ? 0 : e;
  }
  a.raw = w.raw.as<RawCand>();
  a.raw_count = w.raw_count.as<unsigned>();
  a.raw_cap = w.raw_cap;
  a.overflow = w.overflow.as<unsigned>();
  // exact f32 form of the h = 1 prefilter (double)max(pw) - 1.0 >= threshold
  float v = (float)(c.threshold + 1.0);
  if (std::isnan(v)) v = INFINITY;
  for (int it = 0; it < 64 && (double)v - 1.0 >= c.threshold; ++it)
    v = std::nextafter(v, -INFINITY);
  for (int it = 0; it < 64 && !((double)v - 1.0 >= c.threshold); ++it)
    v = std::nextafter(v, INFINITY);
  a.t1 = v;
  return a;
}
GateArgs gate_args(SpecWork &w, uint64_t slot0) {
  GateArgs g{};
  g.qcap = w.qcap;
  g.q1 = w.gq.as<uint32_t>() + slot0 * w.qcap;
  g.q2 = w.gq.as<uint32_t>() + (w.outer_trials + slot0) * w.qcap;
  g.n1 = w.gn.as<unsigned>() + slot0;
  g.n2 = w.gn.as<unsigned>() + w.outer_trials + slot0;
  return g;
}
}  // namespace

// Normalisation scales and harmonic gates of the `ntrials` spectra at slots
// [slot0, slot0 + ntrials) of the outer chunk (d_power/d_psum point at slot0).
int spectrum_gate(const FftPlan &p, const SpecConfig &c, const float *d_power, uint64_t ldp,
                  const double *d_psum, uint32_t npsum, uint64_t ntrials, uint64_t slot0,
                  SpecWork &w, cudaStream_t st) {
  const uint64_t plen = p.M + 1;
  const uint64_t nblocks = (plen + 63) / 64;
  HarmArgs a = harm_args(p, c, d_power, ldp, w);
  GateArgs g = gate_args(w, slot0);
  PSR_CUDA(cudaFuncSetAttribute(k_scales_gate, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)SCG_SMEM));
  dim3 grid((unsigned)((nblocks + SC_G - 1) / SC_G), (unsigned)ntrials);
  k_scales_gate<<<grid, SC_NT, SCG_SMEM, st>>>(a, d_psum, npsum, nblocks,
                                               w.scale.as<float>() + slot0 * w.lds, g);
  PSR_CUDA(cudaGetLastError());
  return PSR_OK;
}

// Exact evaluation of every queued bin of the outer chunk's `ntrials` spectra.
int spectrum_items(const FftPlan &p, const SpecConfig &c, const float *d_power, uint64_t ldp,
                   uint64_t ntrials, SpecWork &w, cudaStream_t st) {
  HarmArgs a = harm_args(p, c, d_power, ldp, w);
  if (a.end[0] == 0) return PSR_OK;
  dim3 grid(HI_CTAS_PER_TRIAL, (unsigned)ntrials);
  if (c.levels == 6)
    k_harm_items<6><<<grid, HI_NT, 0, st>>>(a, gate_args(w, 0));
  else
    k_harm_items<5><<<grid, HI_NT, 0, st>>>(a, gate_args(w, 0));
  PSR_CUDA(cudaGetLastError());
  return PSR_OK;
}

// Sort/dedupe the raw candidates of `ntrials` trials into kept[][max_candidates].
int spectrum_select(const FftPlan &p, const SpecConfig &c, const double *d_trial_dm,
                    uint64_t ntrials, SpecWork &w, psr_candidate *d_kept, unsigned *d_kept_count,
                    cudaStream_t st) {
  SelArgs s{};
  s.raw = w.raw.as<RawCand>();
  s.raw_count = w.raw_count.as<unsigned>();
  s.raw_cap = w.raw_cap;
  s.trial_dm = d_trial_dm;
  s.tol = 1.0 / ((double)p.len * c.tsamp);
  s.max_candidates = c.max_candidates;
  s.kept = d_kept;
  s.kept_count = d_kept_count;
  k_select<<<(unsigned)ntrials, SEL_NT, 0, st>>>(s);
  PSR_CUDA(cudaGetLastError());
  return PSR_OK;
}

}  // namespace psr
