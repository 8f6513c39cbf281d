// K1 unpack (fbank::decode) and K2 RFI masking (rfi::mask) on the device.
//
// Layout: samples are channel-major, row c at c*ld, stored in their integer
// width (u8 for nbits <= 8, u16, f32).  Decisions of rfi::mask depend on the
// reference's sequential f32 sums (rfi/src/lib.rs:35-43, 59-67); every sum
// whose order matters is computed by one thread in reference order, and sums
// that are provably exact (integer samples, total <= 2^24) are computed in
// parallel, which gives the identical f32 value.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "psr_internal.h"

namespace psr {

namespace {

constexpr int UNPACK_TT = 256;  // times per tile
constexpr int UNPACK_TC = 32;   // channels per tile

template <class T>
__global__ void k_unpack(const uint8_t *__restrict__ payload, T *__restrict__ out,
                         uint64_t ns, uint64_t nch, uint64_t ld, int nbits,
                         unsigned long long *err_index) {
  __shared__ T tile[UNPACK_TC][UNPACK_TT + 4];
  const uint64_t t0 = (uint64_t)blockIdx.x * UNPACK_TT;
  const uint64_t c0 = (uint64_t)blockIdx.y * UNPACK_TC;
  for (int idx = threadIdx.x; idx < UNPACK_TT * UNPACK_TC; idx += blockDim.x) {
    int tl = idx / UNPACK_TC, cl = idx % UNPACK_TC;
    uint64_t t = t0 + tl, c = c0 + cl;
    T v = T(0);
    if (t < ns && c < nch) {
      uint64_t i = t * nch + c;
      if constexpr (sizeof(T) == 1) {
        if (nbits == 8) {
          v = payload[i];
        } else {
          // SIGPROC packs low-bit samples LSB first (fbank/src/lib.rs:175-179).
          uint64_t bit = i * (uint64_t)nbits;
          v = (T)((payload[bit >> 3] >> (bit & 7)) & ((1u << nbits) - 1u));
        }
      } else if constexpr (sizeof(T) == 2) {
        v = (T)(payload[2 * i] | ((unsigned)payload[2 * i + 1] << 8));
      } else {
        uint32_t b = (uint32_t)payload[4 * i] | ((uint32_t)payload[4 * i + 1] << 8) |
                     ((uint32_t)payload[4 * i + 2] << 16) | ((uint32_t)payload[4 * i + 3] << 24);
        float f = __uint_as_float(b);
        if (!isfinite(f)) atomicMin(err_index, (unsigned long long)i);
        v = f;
      }
    }
    tile[cl][tl] = v;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < UNPACK_TT * UNPACK_TC; idx += blockDim.x) {
    int cl = idx / UNPACK_TT, tl = idx % UNPACK_TT;
    uint64_t t = t0 + tl, c = c0 + cl;
    if (t < ns && c < nch) out[c * ld + t] = tile[cl][tl];
  }
}

// ------------------------------------------------------------ radix select
// Total-order key of an f32 (Rust f32::total_cmp) as an unsigned integer.
__device__ __forceinline__ uint32_t fkey(float f) {
  uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float fkey_inv(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// Block-wide exact selection of the element of rank r (ascending) among n
// keys key(i); top_shift is the shift of the highest non-constant digit.
// Each warp counts digits in its own histogram (hist holds 32 x 256 slots),
// so few-valued data (4-bit samples) does not serialise on a handful of bins.
template <class KeyFn>
__device__ uint32_t block_select(KeyFn key, uint64_t n, uint64_t r, int top_shift,
                                 unsigned *hist, uint32_t *bcast) {
  const int nw = (int)(blockDim.x + 31) / 32;
  unsigned *mine = hist + (threadIdx.x >> 5) * 256;
  uint32_t prefix = 0, mask = 0;
  for (int shift = top_shift; shift >= 0; shift -= 8) {
    for (int d = threadIdx.x; d < nw * 256; d += blockDim.x) hist[d] = 0;
    __syncthreads();
    for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) {
      uint32_t k = key(i);
      if ((k & mask) == prefix) atomicAdd(&mine[(k >> shift) & 255u], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) {
      unsigned t = 0;
      for (int w = 0; w < nw; ++w) t += hist[w * 256 + d];
      hist[d] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      uint64_t cum = 0;
      uint32_t digit = 255;
      for (int d = 0; d < 256; ++d) {
        if (cum + hist[d] > r) {
          digit = (uint32_t)d;
          break;
        }
        cum += hist[d];
      }
      r -= cum;
      bcast[0] = digit;
      bcast[1] = (uint32_t)(r & 0xffffffffu);
      bcast[2] = (uint32_t)(r >> 32);
    }
    __syncthreads();
    uint32_t digit = bcast[0];
    r = (uint64_t)bcast[1] | ((uint64_t)bcast[2] << 32);
    prefix |= digit << shift;
    mask |= 255u << shift;
    __syncthreads();
  }
  return prefix;
}

__global__ void k_median_f32(const float *__restrict__ v, uint64_t n, float *out) {
  __shared__ unsigned hist[32 * 256];
  __shared__ uint32_t bc[3];
  if (n == 0) {
    if (threadIdx.x == 0) *out = 0.0f;
    return;
  }
  uint32_t k = block_select([&](uint64_t i) { return fkey(v[i]); }, n, n / 2, 24, hist, bc);
  if (threadIdx.x == 0) *out = fkey_inv(k);
}

// Per-channel exact median of the original row (rfi/src/lib.rs:78).
template <class T>
__global__ void k_chan_median(const T *__restrict__ s, uint64_t ns, uint64_t ld,
                              float *__restrict__ med) {
  __shared__ unsigned hist[32 * 256];
  __shared__ uint32_t bc[3];
  const T *row = s + (uint64_t)blockIdx.x * ld;
  uint32_t k;
  if constexpr (sizeof(T) == 1) {
    k = block_select([&](uint64_t i) { return (uint32_t)row[i]; }, ns, ns / 2, 0, hist, bc);
    if (threadIdx.x == 0) med[blockIdx.x] = (float)k;
  } else if constexpr (sizeof(T) == 2) {
    k = block_select([&](uint64_t i) { return (uint32_t)row[i]; }, ns, ns / 2, 8, hist, bc);
    if (threadIdx.x == 0) med[blockIdx.x] = (float)k;
  } else {
    k = block_select([&](uint64_t i) { return fkey(row[i]); }, ns, ns / 2, 24, hist, bc);
    if (threadIdx.x == 0) med[blockIdx.x] = fkey_inv(k);
  }
}

// 8-bit rows: the median from a 256-bin histogram (one pass).  Each row is
// split over MH_SPLIT CTAs; every thread counts into its own 16-bit column
// of a [256][MH_NT] table in shared memory (no atomics, bank = thread / 2),
// the columns are summed per bin and added to the row's global histogram.
constexpr int MH_NT = 128;
constexpr size_t MH_SMEM = 256 * MH_NT * sizeof(uint16_t);

__global__ void __launch_bounds__(MH_NT)
    k_chan_hist_u8(const uint8_t *__restrict__ s, uint64_t ns, uint64_t ld,
                   unsigned *__restrict__ hist) {
  extern __shared__ uint32_t h32[];
  uint16_t *h16 = reinterpret_cast<uint16_t *>(h32);
  const int tid = (int)threadIdx.x;
  for (int i = tid; i < 256 * MH_NT / 2; i += MH_NT) h32[i] = 0u;
  __syncthreads();
  const uint8_t *row = s + (uint64_t)blockIdx.y * ld;
  // this CTA's range [a, b), a a multiple of 16 (rows are 64-byte aligned
  // and padded by >= 64 bytes, so whole 16-byte loads stay in the row)
  const uint64_t per = (((ns + gridDim.x - 1) / gridDim.x) + 15) & ~15ull;
  const uint64_t a = (uint64_t)blockIdx.x * per, b = min(ns, a + per);
  uint16_t *mine = h16 + tid;
  for (uint64_t i = a + (uint64_t)tid * 16; i < b; i += (uint64_t)MH_NT * 16) {
    const uint4 v = __ldg(reinterpret_cast<const uint4 *>(row + i));
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
    const int m = (int)min((uint64_t)16, b - i);
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if (k < m) mine[((w[k >> 2] >> (8 * (k & 3))) & 255u) * MH_NT] += 1;
  }
  __syncthreads();
  for (int bin = tid; bin < 256; bin += MH_NT) {
    const uint16_t *hb = h16 + bin * MH_NT;
    unsigned t = 0;
    for (int j = 0; j < MH_NT; ++j) {
      int k = j + tid;
      if (k >= MH_NT) k -= MH_NT;
      t += hb[k];
    }
    if (t) atomicAdd(&hist[(uint64_t)blockIdx.y * 256 + bin], t);
  }
}

// Element of rank ns / 2 from each row's histogram (one thread per row).
__global__ void k_hist_median(const unsigned *__restrict__ hist, uint64_t nch, uint64_t ns,
                              float *__restrict__ med) {
  const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nch) return;
  const uint64_t r = ns / 2;
  uint64_t cum = 0;
  int d = 255;
  for (int k = 0; k < 256; ++k) {
    cum += hist[c * 256 + k];
    if (cum > r) {
      d = k;
      break;
    }
  }
  med[c] = (float)d;
}

// Exact integer channel totals (for the provably-exact f32 fast path).
template <class T>
__global__ void k_chan_total(const T *__restrict__ s, uint64_t ns, uint64_t ld,
                             unsigned long long *__restrict__ tot) {
  const T *row = s + (uint64_t)blockIdx.y * ld;
  unsigned long long acc = 0;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ns;
       t += (uint64_t)gridDim.x * blockDim.x)
    acc += (unsigned long long)row[t];
  for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(&tot[blockIdx.y], acc);
}

template <class T>
__device__ __forceinline__ float as_f32(T v) {
  return (float)v;
}

// Channel means and variances (rfi/src/lib.rs:35-43), in reference order,
// with the per-sample work taken off the sequential chain: one
// CTA per channel; warps 1.. write the f32 terms of the next segment into a
// shared-memory double buffer while thread 0 adds the current segment's terms
// in reference order.  The chain then costs one FADD latency per sample.
constexpr int PC_NT = 256;
constexpr int PC_SEG = 2048;

template <class T, class Term>
__device__ float pc_sequential_sum(const T *row, uint64_t ns, float *buf, Term term) {
  const uint64_t nseg = (ns + PC_SEG - 1) / PC_SEG;
  float acc = -0.0f;
  constexpr int NP = PC_NT - 32;                 // producer threads
  constexpr int NI = (PC_SEG + NP - 1) / NP;     // samples per producer thread
  auto produce = [&](uint64_t seg, float *dst) {
    const uint64_t t0 = seg * PC_SEG;
    const int cnt = (int)min((uint64_t)PC_SEG, ns - t0);
    float v[NI];
#pragma unroll
    for (int u = 0; u < NI; ++u) {  // all loads issued before any is used
      const int i = (int)threadIdx.x - 32 + u * NP;
      v[u] = i < cnt ? as_f32(row[t0 + i]) : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < NI; ++u) {
      const int i = (int)threadIdx.x - 32 + u * NP;
      if (i < cnt) dst[i] = term(v[u]);
    }
  };
  if (threadIdx.x >= 32) produce(0, buf);
  __syncthreads();
  for (uint64_t seg = 0; seg < nseg; ++seg) {
    float *cur = buf + (seg & 1) * PC_SEG;
    if (threadIdx.x >= 32) {
      if (seg + 1 < nseg) produce(seg + 1, buf + ((seg + 1) & 1) * PC_SEG);
    } else if (threadIdx.x == 0) {
      const int cnt = (int)min((uint64_t)PC_SEG, ns - seg * PC_SEG);
      const float4 *c4 = reinterpret_cast<const float4 *>(cur);
      int i = 0;
#pragma unroll 8
      for (; i + 4 <= cnt; i += 4) {
        const float4 q = c4[i >> 2];
        acc = __fadd_rn(acc, q.x);
        acc = __fadd_rn(acc, q.y);
        acc = __fadd_rn(acc, q.z);
        acc = __fadd_rn(acc, q.w);
      }
      for (; i < cnt; ++i) acc = __fadd_rn(acc, cur[i]);
    }
    __syncthreads();
  }
  return acc;  // valid in thread 0
}

template <class T>
__global__ void __launch_bounds__(PC_NT)
    k_chan_mean_var_pc(const T *__restrict__ s, uint64_t ns, uint64_t ld,
                       const unsigned long long *__restrict__ tot, float *__restrict__ means,
                       float *__restrict__ vars) {
  __shared__ __align__(16) float buf[2 * PC_SEG];
  __shared__ float mean_s;
  const uint64_t c = blockIdx.x;
  const T *row = s + c * ld;
  if (sizeof(T) < 4 && tot[c] <= (1ull << 24)) {
    if (threadIdx.x == 0) mean_s = __fdiv_rn((float)tot[c], (float)ns);
  } else {
    const float sum = pc_sequential_sum(row, ns, buf, [](float x) { return x; });
    if (threadIdx.x == 0) mean_s = __fdiv_rn(sum, (float)ns);
  }
  __syncthreads();
  const float m = mean_s;
  const float acc = pc_sequential_sum(row, ns, buf, [m](float x) {
    const float d = __fsub_rn(x, m);
    return __fmul_rn(d, d);
  });
  if (threadIdx.x == 0) {
    means[c] = m;
    vars[c] = __fdiv_rn(acc, (float)ns);
  }
}

// Reference-order f32 sums of non-negative terms, s = RN(...RN(RN(-0 + t0) +
// t1)... + t_{n-1}), bit for bit, in parallel.  While s stays in one binade
// [2^e, 2^(e+1)) every representable value is a multiple of u = 2^(e-23), so
// s = K u (2^23 <= K < 2^24) and RN(s + t) = (K + inc(t)) u with inc(t) =
// t/u rounded to nearest: the integer part q of t/u plus one when its
// fraction exceeds 1/2.  An exact half (a tie) rounds to even: inc = q +
// ((K + q) mod 2), so it depends on the running K only through its parity,
// and leaves K even.  The parity after a run of terms is therefore either
// P xor c (no tie in the run) or a constant (after its last tie): these maps
// compose, so a warp scans them across its lanes, and the total of a
// 512-term chunk is a known sum plus, when it holds a tie, one bit that
// depends on K's parity at the chunk's start.  t >= 0 makes K monotone; a
// chunk whose total keeps K + total < 2^24 is added at once.  Chunks with a
// binade crossing, a subnormal, infinite or NaN term, or s still 0 or
// subnormal are added term by term in order.
constexpr int ES_L = 512;  // terms per chunk, 16 per lane

// One term at unit u = 2^(e - 23): inc = q (+1 above the half), kind 0;
// kind 1: an exact half (inc = q, the rounding bit comes from K's parity);
// kind 2: a term the binade arithmetic does not cover.
__device__ __forceinline__ int es_term(float t, int e, unsigned long long &inc) {
  const uint32_t b = __float_as_uint(t);
  const int be = (int)((b >> 23) & 0xff);
  inc = 0;
  if (be == 0 || be == 255) return (b & 0x7fffffffu) != 0u ? 2 : 0;  // +-0 adds nothing
  const uint32_t mt = (b & 0x7fffffu) | 0x800000u;
  const int sh = (be - 150) - (e - 23);  // t / u = mt 2^sh
  if (sh >= 0) {
    // t >= 2^23 u > 2^e would leave the binade: count it as 2^40 units
    // (any such term fails the K + total < 2^24 test; no 64-bit overflow)
    inc = sh >= 24 ? (1ull << 40) : ((unsigned long long)mt << sh);
    return 0;
  }
  if (sh <= -25) return 0;  // below half a unit
  const int r = -sh;
  const uint32_t rem = mt & ((1u << r) - 1u), half = 1u << (r - 1);
  inc = (unsigned long long)(mt >> r) + (rem > half ? 1ull : 0ull);
  return rem == half ? 1 : 0;
}

// A warp's chunk at unit u: total(P0) = base + (tie ? P0 ^ bit : 0) for K's
// parity P0 at the chunk's start; special: the chunk must go term by term.
struct EsChunk {
  unsigned long long base;
  int bit;
  bool tie, special;
};

template <int PER>
__device__ __forceinline__ EsChunk es_chunk_warp(const float (&t)[PER], int e, int lane) {
  // lane map: constant (after a tie in the lane) or xor
  bool lc = false, lsp = false;
  uint32_t lv = 0;
  unsigned long long lsum = 0;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    unsigned long long inc;
    const int k = es_term(t[j], e, inc);
    lsum += inc;
    if (k == 2) {
      lsp = true;
    } else if (k == 1) {
      lc = true;
      lv = 0;
    } else {
      lv ^= (uint32_t)inc & 1u;
    }
  }
  EsChunk c;
  c.bit = 0;
  c.tie = __any_sync(0xffffffffu, lc);
  c.special = __any_sync(0xffffffffu, lsp);
  if (!c.tie) {  // (most chunks) the total does not depend on K
#pragma unroll
    for (int o = 16; o; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    c.base = lsum;
    return c;
  }
  // inclusive scan of the maps, then the map from the chunk start to this lane
  bool ic = lc;
  uint32_t v = lv;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const bool pic = __shfl_up_sync(0xffffffffu, ic, o);
    const uint32_t pv = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) {
      v = ic ? v : (pv ^ v);
      ic = ic || pic;
    }
  }
  bool conc = __shfl_up_sync(0xffffffffu, ic, 1);
  uint32_t P = __shfl_up_sync(0xffffffffu, v, 1);
  if (lane == 0) {
    conc = false;
    P = 0;
  }
  // conc: P is K's parity; otherwise K's parity is P0 ^ P
  unsigned long long base = 0;
  int fb = -1;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    unsigned long long inc;
    const int k = es_term(t[j], e, inc);
    if (k == 1) {
      if (conc) {
        base += inc + ((P + (uint32_t)inc) & 1u);
      } else {  // the chunk's first tie: its bit waits for P0
        base += inc;
        fb = (int)((P ^ (uint32_t)inc) & 1u);
      }
      P = 0;
      conc = true;
    } else if (k == 0) {
      base += inc;
      P ^= (uint32_t)inc & 1u;
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) base += __shfl_xor_sync(0xffffffffu, base, o);
  const unsigned fm = __ballot_sync(0xffffffffu, fb >= 0);
  c.base = base;
  c.bit = fm ? __shfl_sync(0xffffffffu, fb, __ffs(fm) - 1) : 0;
  return c;
}

// Lane l's 16 consecutive samples of chunk g of a step: one or two aligned
// 16-byte loads (rows start 64-element aligned; only issued for samples below
// ns, whose 16-sample run then ends inside the row's padding).
template <class T>
struct EsRaw {
  static constexpr int W = 16 * (int)sizeof(T) / 16;
  uint4 r[W];
  __device__ __forceinline__ void load(const T *p, bool ok) {
#pragma unroll
    for (int k = 0; k < W; ++k)
      r[k] = ok ? __ldg(reinterpret_cast<const uint4 *>(p) + k) : make_uint4(0u, 0u, 0u, 0u);
  }
  __device__ __forceinline__ float at(int j) const {
    if constexpr (sizeof(T) == 1) {
      const uint32_t w = (r[0].x * (j >> 2 == 0)) | (r[0].y * (j >> 2 == 1)) |
                         (r[0].z * (j >> 2 == 2)) | (r[0].w * (j >> 2 == 3));
      return (float)((w >> (8 * (j & 3))) & 255u);
    } else {
      const uint4 &q = r[j >> 3];
      const int e = (j >> 1) & 3;
      const uint32_t w = e == 0 ? q.x : (e == 1 ? q.y : (e == 2 ? q.z : q.w));
      return (float)((w >> (16 * (j & 1))) & 65535u);
    }
  }
};

constexpr int ES_G = 16;  // chunks per step = warps per CTA

// One CTA of ES_G warps per channel: warp w holds chunk w of every step of
// ES_G chunks (its samples prefetched a step ahead), computes the chunk's
// total at the binade of the running s, and the CTA adds the longest run of
// chunks that stays in the binade (each tie's rounding bit from the running
// parity); a chunk that cannot be is added term by term, in order, by
// thread 0.  Returns s in every thread.
struct EsShared {
  float stage[ES_L];
  unsigned long long tot[ES_G];
  int tie[ES_G], bit[ES_G], special[ES_G];
  float s;
};

template <class T, class Term>
__device__ float exact_seq_sum_cta(const T *__restrict__ row, uint64_t ns, Term term,
                                   EsShared &sh) {
  const int lane = (int)(threadIdx.x & 31), g = (int)(threadIdx.x >> 5);
  constexpr int PER = ES_L / 32;
  constexpr uint64_t STEP = (uint64_t)ES_G * ES_L;
  if (threadIdx.x == 0) sh.s = -0.0f;
  EsRaw<T> raw, nxt;
  {
    const uint64_t i0 = (uint64_t)g * ES_L + (uint64_t)lane * PER;
    raw.load(row + i0, i0 < ns);
  }
  __syncthreads();
  for (uint64_t c0 = 0; c0 < ns; c0 += STEP) {
    const uint64_t i0 = c0 + (uint64_t)g * ES_L + (uint64_t)lane * PER;
    nxt.load(row + i0 + STEP, i0 + STEP < ns);
    float t[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j) t[j] = i0 + j < ns ? term(raw.at(j)) : 0.0f;
    const int nchunk = (int)min((uint64_t)ES_G, (ns - c0 + ES_L - 1) / ES_L);
    int g0 = 0;
    while (g0 < nchunk) {  // g0 and sh.s are uniform across the CTA
      const float s = sh.s;
      const uint32_t sb = __float_as_uint(s);
      const int se = (int)((sb >> 23) & 0xff);
      int g1 = g0;
      if (se > 0 && se < 255 && !(sb >> 31)) {
        const int e = se - 127;
        if (g >= g0) {  // warp-uniform
          const EsChunk ck = es_chunk_warp<PER>(t, e, lane);
          if (lane == 0) {
            sh.tot[g] = ck.base;
            sh.tie[g] = ck.tie ? 1 : 0;
            sh.bit[g] = ck.bit;
            sh.special[g] = ck.special ? 1 : 0;
          }
        }
        __syncthreads();
        unsigned long long acc = (sb & 0x7fffffu) | 0x800000u;
        bool stop = false;
#pragma unroll
        for (int k = 0; k < ES_G; ++k) {
          if (k >= g0 && k < nchunk && !stop) {
            // a chunk with a tie: its first tie rounds by K's parity here
            const uint32_t rb = ((uint32_t)acc ^ (uint32_t)sh.bit[k]) & 1u;
            const unsigned long long tk = sh.tot[k] + (sh.tie[k] ? rb : 0u);
            if (sh.special[k] || acc + tk >= (1ull << 24)) {
              stop = true;
            } else {
              acc += tk;
              g1 = k + 1;
            }
          }
        }
        __syncthreads();  // every thread has read sh.s, sh.tot and sh.tie
        if (g1 > g0 && threadIdx.x == 0)
          sh.s = __uint_as_float(((uint32_t)(e + 127) << 23) | ((uint32_t)acc & 0x7fffffu));
      }
      if (g1 == g0) {  // chunk g0 term by term
        if (g == g0)
#pragma unroll
          for (int j = 0; j < PER; ++j) sh.stage[lane * PER + j] = t[j];
        __syncthreads();
        if (threadIdx.x == 0) {
          float a = sh.s;
          const int cnt = (int)min((uint64_t)ES_L, ns - (c0 + (uint64_t)g0 * ES_L));
          for (int i = 0; i < cnt; ++i) a = __fadd_rn(a, sh.stage[i]);
          sh.s = a;
        }
        g1 = g0 + 1;
      }
      __syncthreads();  // sh.s updated
      g0 = g1;
    }
    raw = nxt;
  }
  return sh.s;
}

// Channel means and variances (rfi/src/lib.rs:35-43) for integer samples:
// one warp per channel, the exact parallel reference-order sums above (the
// mean straight from the exact integer total while it is below 2^24).
template <class T>
__global__ void __launch_bounds__(32 * ES_G)
    k_chan_mean_var_ex(const T *__restrict__ s, uint64_t ns, uint64_t ld,
                       const unsigned long long *__restrict__ tot, float *__restrict__ means,
                       float *__restrict__ vars) {
  __shared__ EsShared sh;
  const uint64_t c = blockIdx.x;
  const T *row = s + c * ld;
  float m;
  if (tot[c] <= (1ull << 24)) {
    m = __fdiv_rn((float)tot[c], (float)ns);
  } else {
    m = __fdiv_rn(exact_seq_sum_cta(row, ns, [](float x) { return x; }, sh), (float)ns);
    __syncthreads();  // sh is reused below
  }
  const float acc = exact_seq_sum_cta(row, ns, [m](float x) {
    const float d = __fsub_rn(x, m);
    return __fmul_rn(d, d);
  }, sh);
  if (threadIdx.x == 0) {
    means[c] = m;
    vars[c] = __fdiv_rn(acc, (float)ns);
  }
}

// Per-(channel, block) sequential f32 sums (rfi/src/lib.rs:62-64).
template <class T>
__global__ void k_block_sums(const T *__restrict__ s, uint64_t ns, uint64_t ld,
                             uint64_t nch, uint64_t bs, uint64_t blocks_n,
                             float *__restrict__ bsum) {
  uint64_t id = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= nch * blocks_n) return;
  uint64_t c = id / blocks_n, b = id % blocks_n;
  uint64_t start = b * bs, end = min(start + bs, ns);
  const T *row = s + c * ld;
  float acc = -0.0f;
  for (uint64_t t = start; t < end; ++t) acc = __fadd_rn(acc, as_f32(row[t]));
  bsum[c * blocks_n + b] = acc;
}

// rfi::outliers (rfi/src/lib.rs:13-22) for one vector, inside one block.
__device__ void block_outliers(const float *v, uint64_t n, float threshold,
                               float *dev_scratch, unsigned char *flags,
                               unsigned *hist, uint32_t *bc) {
  float center = 0.0f;
  if (n > 0) {
    uint32_t k = block_select([&](uint64_t i) { return fkey(v[i]); }, n, n / 2, 24, hist, bc);
    center = fkey_inv(k);
  }
  for (uint64_t i = threadIdx.x; i < n; i += blockDim.x)
    dev_scratch[i] = fabsf(__fsub_rn(v[i], center));
  __syncthreads();
  float mad = 0.0f;
  if (n > 0) {
    uint32_t k = block_select([&](uint64_t i) { return fkey(dev_scratch[i]); }, n, n / 2, 24,
                              hist, bc);
    mad = fkey_inv(k);
  }
  float scale = fmaxf(fmaxf(__fmul_rn(1.4826f, mad), __fmul_rn(fabsf(center), 1e-4f)), 1e-6f);
  float lim = __fmul_rn(threshold, scale);
  for (uint64_t i = threadIdx.x; i < n; i += blockDim.x)
    flags[i] = fabsf(__fsub_rn(v[i], center)) > lim ? 1 : 0;
  __syncthreads();
}

// Channel decision (rfi/src/lib.rs:44-48); writes chbad[] and active count.
__global__ void k_channel_decide(const float *means, const float *vars, uint64_t nch,
                                 float threshold, float *scratch, unsigned char *f1,
                                 unsigned char *f2, unsigned char *chbad,
                                 unsigned long long *active) {
  __shared__ unsigned hist[32 * 256];
  __shared__ uint32_t bc[3];
  block_outliers(means, nch, threshold, scratch, f1, hist, bc);
  block_outliers(vars, nch, threshold, scratch, f2, hist, bc);
  for (uint64_t c = threadIdx.x; c < nch; c += blockDim.x)
    chbad[c] = (f1[c] || f2[c] || vars[c] < 1e-12f) ? 1 : 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long a = 0;
    for (uint64_t c = 0; c < nch; ++c) a += chbad[c] ? 0 : 1;
    *active = a;
  }
}

// Block means over good channels in channel order (rfi/src/lib.rs:55-69).
__global__ void k_block_means(const float *bsum, const unsigned char *chbad, uint64_t nch,
                              uint64_t ns, uint64_t bs, uint64_t blocks_n,
                              const unsigned long long *active, float *bmeans) {
  uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= blocks_n) return;
  float sum = 0.0f;
  for (uint64_t c = 0; c < nch; ++c)
    if (!chbad[c]) sum = __fadd_rn(sum, bsum[c * blocks_n + b]);
  uint64_t start = b * bs, end = min(start + bs, ns);
  unsigned long long a = *active;
  if (a < 1) a = 1;
  bmeans[b] = __fdiv_rn(sum, (float)((end - start) * a));
}

__global__ void k_block_decide(const float *bmeans, uint64_t blocks_n, float threshold,
                               float *scratch, unsigned char *blkbad) {
  __shared__ unsigned hist[32 * 256];
  __shared__ uint32_t bc[3];
  block_outliers(bmeans, blocks_n, threshold, scratch, blkbad, hist, bc);
}

// Replace masked samples with the channel median (rfi/src/lib.rs:76-89).
template <class T>
__global__ void k_fill(T *__restrict__ s, uint64_t ns, uint64_t ld, uint64_t bs,
                       const unsigned char *__restrict__ chbad,
                       const unsigned char *__restrict__ blkbad,
                       const float *__restrict__ med) {
  uint64_t c = blockIdx.y;
  T typical = (T)med[c];
  bool whole = chbad[c] != 0;
  T *row = s + c * ld;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ns;
       t += (uint64_t)gridDim.x * blockDim.x)
    if (whole || blkbad[t / bs]) row[t] = typical;
}

}  // namespace

int DeviceObs::alloc(cudaStream_t st) {
  ld = ((ns + 64 + 63) / 64) * 64;
  size_t bytes = (size_t)ld * nch * sample_bytes(kind) + 256;
  PSR_TRY(samples.ensure(bytes));
  // on the stream that fills the samples next: a plain cudaMemset runs on the
  // legacy default stream, which does not order against non-blocking streams
  PSR_CUDA(cudaMemsetAsync(samples.p, 0, bytes, st));
  return PSR_OK;
}

int launch_unpack(const DeviceObs &o, unsigned long long *d_err, cudaStream_t st) {
  dim3 grid((unsigned)((o.ns + UNPACK_TT - 1) / UNPACK_TT),
            (unsigned)((o.nch + UNPACK_TC - 1) / UNPACK_TC));
  const uint8_t *p = o.payload.as<uint8_t>();
  switch (o.kind) {
    case SAMPLE_U8:
      k_unpack<uint8_t><<<grid, 256, 0, st>>>(p, o.samples.as<uint8_t>(), o.ns, o.nch, o.ld,
                                              (int)o.h.nbits, d_err);
      break;
    case SAMPLE_U16:
      k_unpack<uint16_t><<<grid, 256, 0, st>>>(p, o.samples.as<uint16_t>(), o.ns, o.nch, o.ld,
                                               (int)o.h.nbits, d_err);
      break;
    default:
      k_unpack<float><<<grid, 256, 0, st>>>(p, o.samples.as<float>(), o.ns, o.nch, o.ld,
                                            (int)o.h.nbits, d_err);
  }
  PSR_CUDA(cudaGetLastError());
  return PSR_OK;
}

int launch_median_f32(const float *d_vals, uint64_t n, float *d_out, unsigned int *,
                      cudaStream_t st) {
  k_median_f32<<<1, 1024, 0, st>>>(d_vals, n, d_out);
  PSR_CUDA(cudaGetLastError());
  return PSR_OK;
}

template <class T>
static int rfi_enqueue_t(DeviceObs &o, uint64_t bs, float thr, RfiWork &w, cudaStream_t st) {
  const uint64_t nch = o.nch, ns = o.ns;
  const uint64_t blocks_n = (ns + bs - 1) / bs;
  w.blocks_n = blocks_n;
  PSR_TRY(w.means.ensure(nch * 4));
  PSR_TRY(w.vars.ensure(nch * 4));
  PSR_TRY(w.med.ensure(nch * 4));
  PSR_TRY(w.bsum.ensure(nch * blocks_n * 4));
  PSR_TRY(w.bmeans.ensure(blocks_n * 4));
  PSR_TRY(w.chbad.ensure(nch));
  PSR_TRY(w.blkbad.ensure(blocks_n));
  PSR_TRY(w.scratch.ensure(std::max(nch, blocks_n) * 4));
  PSR_TRY(w.flags.ensure(2 * nch));
  PSR_TRY(w.hist.ensure(nch * 8 + 8));
  T *s = o.samples.as<T>();
  unsigned long long *tot = w.hist.as<unsigned long long>();
  PSR_CUDA(cudaMemsetAsync(tot, 0, nch * 8 + 8, st));
  if (sizeof(T) < 4) {
    dim3 g((unsigned)std::min<uint64_t>((ns + 255) / 256, 64), (unsigned)nch);
    k_chan_total<T><<<g, 256, 0, st>>>(s, ns, o.ld, tot);
  }
  if constexpr (sizeof(T) < 4)
    k_chan_mean_var_ex<T><<<(unsigned)nch, 32 * ES_G, 0, st>>>(s, ns, o.ld, tot, w.means.as<float>(),
                                                       w.vars.as<float>());
  else
    k_chan_mean_var_pc<T><<<(unsigned)nch, PC_NT, 0, st>>>(s, ns, o.ld, tot,
                                                          w.means.as<float>(),
                                                          w.vars.as<float>());
  k_block_sums<T><<<(unsigned)((nch * blocks_n + 127) / 128), 128, 0, st>>>(
      s, ns, o.ld, nch, bs, blocks_n, w.bsum.as<float>());
  if constexpr (sizeof(T) == 1) {
    // per-thread counts stay below 2^16: at most ns / nsplit / MH_NT + 16
    const uint64_t nsplit = std::max<uint64_t>(16, (ns + 60000ull * MH_NT - 1) / (60000ull * MH_NT));
    PSR_TRY(w.mhist.ensure(nch * 256 * 4));
    PSR_CUDA(cudaMemsetAsync(w.mhist.p, 0, nch * 256 * 4, st));
    PSR_CUDA(cudaFuncSetAttribute(k_chan_hist_u8, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)MH_SMEM));
    k_chan_hist_u8<<<dim3((unsigned)nsplit, (unsigned)nch), MH_NT, MH_SMEM, st>>>(
        s, ns, o.ld, w.mhist.as<unsigned>());
    k_hist_median<<<(unsigned)((nch + 127) / 128), 128, 0, st>>>(w.mhist.as<unsigned>(), nch, ns,
                                                                 w.med.as<float>());
  } else {
    k_chan_median<T><<<(unsigned)nch, 512, 0, st>>>(s, ns, o.ld, w.med.as<float>());
  }
  unsigned char *fl = w.flags.as<unsigned char>();
  k_channel_decide<<<1, 1024, 0, st>>>(w.means.as<float>(), w.vars.as<float>(), nch, thr,
                                       w.scratch.as<float>(), fl, fl + nch,
                                       w.chbad.as<unsigned char>(), tot + nch);
  k_block_means<<<(unsigned)((blocks_n + 127) / 128), 128, 0, st>>>(
      w.bsum.as<float>(), w.chbad.as<unsigned char>(), nch, ns, bs, blocks_n, tot + nch,
      w.bmeans.as<float>());
  k_block_decide<<<1, 1024, 0, st>>>(w.bmeans.as<float>(), blocks_n, thr,
                                     w.scratch.as<float>(), w.blkbad.as<unsigned char>());
  dim3 gf((unsigned)std::min<uint64_t>((ns + 255) / 256, 256), (unsigned)nch);
  k_fill<T><<<gf, 256, 0, st>>>(s, ns, o.ld, bs, w.chbad.as<unsigned char>(),
                                w.blkbad.as<unsigned char>(), w.med.as<float>());
  PSR_CUDA(cudaGetLastError());
  return PSR_OK;
}

template <class T>
static int channel_stats_t(const DeviceObs &o, RfiWork &w, cudaStream_t st) {
  const uint64_t nch = o.nch, ns = o.ns;
  PSR_TRY(w.means.ensure(nch * 4));
  PSR_TRY(w.vars.ensure(nch * 4));
  PSR_TRY(w.hist.ensure(nch * 8 + 8));
  const T *s = o.samples.as<T>();
  unsigned long long *tot = w.hist.as<unsigned long long>();
  PSR_CUDA(cudaMemsetAsync(tot, 0, nch * 8 + 8, st));
  if constexpr (sizeof(T) < 4) {
    dim3 g((unsigned)std::min<uint64_t>((ns + 255) / 256, 64), (unsigned)nch);
    k_chan_total<T><<<g, 256, 0, st>>>(s, ns, o.ld, tot);
    k_chan_mean_var_ex<T><<<(unsigned)nch, 32 * ES_G, 0, st>>>(s, ns, o.ld, tot, w.means.as<float>(),
                                                       w.vars.as<float>());
  } else {
    k_chan_mean_var_pc<T><<<(unsigned)nch, PC_NT, 0, st>>>(s, ns, o.ld, tot,
                                                          w.means.as<float>(),
                                                          w.vars.as<float>());
  }
  PSR_CUDA(cudaGetLastError());
  return PSR_OK;
}

int rfi_channel_stats(const DeviceObs &o, float *means, float *variances, cudaStream_t st) {
  RfiWork w;
  switch (o.kind) {
    case SAMPLE_U8: PSR_TRY(channel_stats_t<uint8_t>(o, w, st)); break;
    case SAMPLE_U16: PSR_TRY(channel_stats_t<uint16_t>(o, w, st)); break;
    default: PSR_TRY(channel_stats_t<float>(o, w, st));
  }
  PSR_CUDA(cudaMemcpyAsync(means, w.means.p, o.nch * 4, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaMemcpyAsync(variances, w.vars.p, o.nch * 4, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  return PSR_OK;
}

int rfi_enqueue(DeviceObs &o, uint64_t bs, float thr, RfiWork &w, cudaStream_t st) {
  if (bs == 0 || !(thr > 0.0f) || !std::isfinite(thr)) {
    set_error("rfi::mask: block_samples > 0 and a finite positive threshold are required");
    return PSR_EINVAL;
  }
  switch (o.kind) {
    case SAMPLE_U8: return rfi_enqueue_t<uint8_t>(o, bs, thr, w, st);
    case SAMPLE_U16: return rfi_enqueue_t<uint16_t>(o, bs, thr, w, st);
    default: return rfi_enqueue_t<float>(o, bs, thr, w, st);
  }
}

int rfi_collect(const DeviceObs &o, uint64_t bs, RfiWork &w, cudaStream_t st, RfiResult &res) {
  std::vector<unsigned char> ch(o.nch), bl(w.blocks_n);
  PSR_CUDA(cudaMemcpyAsync(ch.data(), w.chbad.p, o.nch, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaMemcpyAsync(bl.data(), w.blkbad.p, w.blocks_n, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  res.channels.clear();
  res.blocks.clear();
  for (uint64_t c = 0; c < o.nch; ++c)
    if (ch[c]) res.channels.push_back(c);
  for (uint64_t b = 0; b < w.blocks_n; ++b)
    if (bl[b]) res.blocks.push_back(b);
  // rfi/src/lib.rs:75-94
  uint64_t count = res.channels.size() * o.ns;
  uint64_t good = o.nch - res.channels.size();
  for (uint64_t b : res.blocks) {
    uint64_t start = b * bs, end = std::min(start + bs, o.ns);
    count += (end - start) * good;
  }
  res.masked_fraction = (double)count / (double)(o.nch * o.ns);
  return PSR_OK;
}

}  // namespace psr
