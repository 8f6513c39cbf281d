// K3 incoherent dedispersion (dedisperse::apply, dedisperse/src/lib.rs:61-90,
// run for many trials as in the CLI loop cli/src/main.rs:462-469).
//
// out[trial][t] = sum_c data[c][t + delay[trial][c]],  t in [0, n).
//
// Integer samples (u8): every partial sum is an integer below 2^16, so the
// reference's channel-ordered f32 sum is exact and any summation order gives
// the bit-identical value.  The fast kernel stages a tile of every channel
// row into shared memory with TMA bulk copies (cp.async.bulk + mbarrier,
// double buffered), and each thread accumulates four sample words (16
// samples, words tl + 256 k of the tile) for a block of trials in packed
// 2 x u16 lanes (samples of <= 4 bits first in 4 x u8 lanes, widened once per
// group of channels).  Consecutive trials whose delay for a channel falls in
// the same aligned word reuse the loaded words (CTA-uniform test) and only
// shift them again.
//
// Everything else (f32 samples, or integer sums that could exceed 2^16) uses
// a kernel that adds channels in reference order in f32.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cstring>
#include <type_traits>
#include <vector>

#include "psr_internal.h"

namespace psr {
namespace {

constexpr int DD_NT = 256;              // threads per CTA
constexpr int DD_TPT = 16;              // samples per thread
constexpr int DD_TT = DD_NT * DD_TPT;   // samples per tile (4096)
constexpr int DD_DB = 8;                // trials per CTA (16-bit lanes only)
constexpr int DD_DB8 = 8;               // trials per CTA with 8-bit lanes (128 registers)
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
// Run by warp 0: lane i stages row c0+i.  The delay of trial d0 + d and
// channel c is delays[min(d0 + d, ntrials - 1) * dstride + c] (global memory,
// or the CTA's block preloaded in shared memory with d0 = 0, ntrials = DB).
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
template <bool BYTE_LANES, int DB, bool PRELOAD>
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

  // preload: the CTA's [DB][nch] block of delays is copied once into shared
  // memory after the row buffers, so that issuing a stage (between chunks,
  // while the other warps wait at the barrier) reads no global memory.
  auto issue = [&](int k, int b) {
    if constexpr (PRELOAD)
      issue_stage<DB>(s, ld, ns, nch, nch,
                      reinterpret_cast<const uint32_t *>(smem + 2 * bstride), DB, 0, t0,
                      (uint64_t)k * cc, cc, smem + b * bstride, rowcap, &info[b], &bars[b],
                      arm_only);
    else
      issue_stage<DB>(s, ld, ns, nch, dstride, delays, ntrials, d0, t0, (uint64_t)k * cc, cc,
                      smem + b * bstride, rowcap, &info[b], &bars[b], arm_only);
  };
  if constexpr (PRELOAD) {
    uint32_t *dly = reinterpret_cast<uint32_t *>(smem + 2 * bstride);
    const unsigned nc = (unsigned)nch;  // DB * nch <= 4096 (16 KB) when preloaded
    for (unsigned i = tl; i < DB * nc; i += DD_NT) {
      const unsigned d = i / nc, c = i - d * nc;
      const uint64_t tr = d0 + d < ntrials ? d0 + d : ntrials - 1;
      dly[i] = delays[tr * dstride + c];
    }
  }
  if (tl == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tl < 32) {
    issue(0, 0);
    if (nchunks > 1) issue(1, 1);
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
      // Thread tl owns words tl + 256 k (k < 4) of the tile.  A trial's row
      // offset `off` (bytes, CTA-uniform) selects words w = off >> 2 onward,
      // shifted right by (off & 3) bytes.  Delays grow by 0 or 1 sample from
      // one trial to the next, so consecutive trials mostly share w: the
      // loaded words are kept and only re-shifted.  Lane d < DB reads trial
      // d's offset; the ballots of "offset changed" and "word changed"
      // against trial d - 1 are warp-uniform bit masks and the offsets are
      // broadcast by shuffles, so every branch below is uniform by
      // construction.
      const uint32_t *row = reinterpret_cast<const uint32_t *>(buf + (size_t)r * rowcap) + tl;
      const int lane = tl & 31;
      const int myoff = info[b].off[r][lane < DB ? lane : DB - 1];
      const int prevoff = __shfl_up_sync(0xffffffffu, myoff, 1);
      const unsigned chg =
          __ballot_sync(0xffffffffu, lane < DB && (lane == 0 || myoff != prevoff));
      const unsigned wchg =
          __ballot_sync(0xffffffffu, lane < DB && (lane == 0 || (myoff >> 2) != (prevoff >> 2)));
      uint32_t a0 = 0, a1 = 0, a2 = 0, a3 = 0, b0 = 0, b1 = 0, b2 = 0, b3 = 0;
      uint32_t x0 = 0, x1 = 0, x2 = 0, x3 = 0;
      // 16-bit lanes: the shifted words split into sample pairs once per
      // offset change, not once per trial
      uint32_t y[BYTE_LANES ? 1 : 8];
#pragma unroll
      for (int i = 0; i < (BYTE_LANES ? 1 : 8); ++i) y[i] = 0;
#pragma unroll
      for (int d = 0; d < DB; ++d) {
        if (chg & (1u << d)) {
          const int off = __shfl_sync(0xffffffffu, myoff, d);
          if (wchg & (1u << d)) {
            const uint32_t *p = row + (off >> 2);
            a0 = p[0];
            b0 = p[1];
            a1 = p[256];
            b1 = p[257];
            a2 = p[512];
            b2 = p[513];
            a3 = p[768];
            b3 = p[769];
          }
          const unsigned sh = (unsigned)(off & 3) * 8u;
          x0 = __funnelshift_r(a0, b0, sh);
          x1 = __funnelshift_r(a1, b1, sh);
          x2 = __funnelshift_r(a2, b2, sh);
          x3 = __funnelshift_r(a3, b3, sh);
          if constexpr (!BYTE_LANES) {
            y[0] = __byte_perm(x0, 0, 0x4140);
            y[1] = __byte_perm(x0, 0, 0x4342);
            y[2] = __byte_perm(x1, 0, 0x4140);
            y[3] = __byte_perm(x1, 0, 0x4342);
            y[4] = __byte_perm(x2, 0, 0x4140);
            y[5] = __byte_perm(x2, 0, 0x4342);
            y[6] = __byte_perm(x3, 0, 0x4140);
            y[7] = __byte_perm(x3, 0, 0x4342);
          }
        }
        if constexpr (BYTE_LANES) {
          acc8[d][0] += x0;
          acc8[d][1] += x1;
          acc8[d][2] += x2;
          acc8[d][3] += x3;
        } else {
#pragma unroll
          for (int i = 0; i < 8; ++i) acc[d][i] += y[i];
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
      issue(k + 2, b);
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

  // Word k of this thread holds samples t0 + 4 (tl + 256 k) + {0, 1, 2, 3}:
  // acc[d][2k] their first two (16-bit lanes), acc[d][2k + 1] the last two.
#pragma unroll
  for (int d = 0; d < DB; ++d) {
    const uint64_t tr = d0 + d;
    unsigned long long local = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint64_t tb = t0 + 4 * ((uint64_t)tl + 256 * k);
      const uint32_t p = acc[d][2 * k], q = acc[d][2 * k + 1];
      const float v[4] = {(float)(p & 0xffffu), (float)(p >> 16), (float)(q & 0xffffu),
                          (float)(q >> 16)};
      if (tb + 4 <= n) {
        local += (p & 0xffffu) + (p >> 16) + (q & 0xffffu) + (q >> 16);
      } else {
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (tb + i < n) local += (unsigned)v[i];
      }
      if (tr < ntrials) {
        // Channel groups after the first add their (integer) partial sums to
        // the earlier groups' in f32: exact while every sum stays below 2^24.
        float *dst = out + tr * ldo + tb;
        if (tb + 4 <= n) {
          float4 w = make_float4(v[0], v[1], v[2], v[3]);
          if (accumulate) {
            const float4 o = *reinterpret_cast<const float4 *>(dst);
            w.x += o.x;
            w.y += o.y;
            w.z += o.z;
            w.w += o.w;
          }
          *reinterpret_cast<float4 *>(dst) = w;
        } else {
          for (int i = 0; i < 4; ++i)
            if (tb + i < n) dst[i] = accumulate ? dst[i] + v[i] : v[i];
        }
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

// ---------------------------------------------------------------------------
// Subband reuse (u8 samples, 16-bit lanes).  Channels are taken in subbands
// of G adjacent channels.  For one block of SB_TB consecutive trials, the
// delays of a subband's channels relative to its smallest delay form a
// pattern; trials that share a pattern share the subband's partial series
// up to a shift.  The plan (host, per block and subband) lists the distinct
// patterns.  Stage A forms each pattern's partial sum over the tile (plus
// the shift range) once in shared memory; stage B adds it, shifted, into
// every trial that uses it.  A subband whose patterns do not repeat enough to
// pay for stage A is added channel by channel (direct).  Every sum is an
// integer below 2^16 in its lane, so the result is bit-identical to the
// reference's channel-ordered f32 sum.
constexpr int SB_TB = 8;    // trials per CTA
constexpr int SB_PMAX = 4;  // patterns per subband held in shared memory
constexpr int SB_GMAX = 8;

struct SbEntry {
  int32_t dref_min;               // smallest subband reference delay in the block
  uint8_t npat, pad0, pad1, pad2;  // npat = 0: direct
  uint8_t pid[SB_TB];             // pattern of each trial
  uint16_t roff[SB_TB];           // reference delay - dref_min, per trial
  uint16_t lo[SB_PMAX], hi[SB_PMAX];  // roff range of each pattern's trials
  uint16_t rel[SB_PMAX][SB_GMAX];     // channel delay - reference delay
};
static_assert(sizeof(SbEntry) == 112, "plan entry layout");

// acc (16-bit lanes: acc[i] = samples 2i | 2i+1 << 16) += the 16 bytes of
// `row` starting at byte `off` (thread's own 16 samples: off includes 16 tl).
__device__ __forceinline__ void add_bytes16(const uint4 *row16, int off, uint32_t *acc) {
  const int q = off >> 4, o = off & 15;
  const uint4 lo = row16[q], hi = row16[q + 1];
  uint32_t w0 = lo.x, w1 = lo.y, w2 = lo.z, w3 = lo.w, w4 = hi.x, w5 = hi.y, w6 = hi.z,
           w7 = hi.w;
  if (o & 8) {
    w0 = w2; w1 = w3; w2 = w4; w3 = w5; w4 = w6; w5 = w7;
  }
  if (o & 4) {
    w0 = w1; w1 = w2; w2 = w3; w3 = w4; w4 = w5;
  }
  const unsigned sh = (unsigned)(o & 3) * 8u;
  const uint32_t x0 = __funnelshift_r(w0, w1, sh), x1 = __funnelshift_r(w1, w2, sh),
                 x2 = __funnelshift_r(w2, w3, sh), x3 = __funnelshift_r(w3, w4, sh);
  acc[0] += __byte_perm(x0, 0, 0x4140);
  acc[1] += __byte_perm(x0, 0, 0x4342);
  acc[2] += __byte_perm(x1, 0, 0x4140);
  acc[3] += __byte_perm(x1, 0, 0x4342);
  acc[4] += __byte_perm(x2, 0, 0x4140);
  acc[5] += __byte_perm(x2, 0, 0x4342);
  acc[6] += __byte_perm(x3, 0, 0x4140);
  acc[7] += __byte_perm(x3, 0, 0x4342);
}

// acc += 16 u16 samples of `pb` starting at sample j (any j >= 0).
__device__ __forceinline__ void add_u16x16(const uint16_t *pb, int j, uint32_t *acc) {
  const int w = j >> 1;  // first word
  const uint4 *p4 = reinterpret_cast<const uint4 *>(pb) + (w >> 2);
  const uint4 a = p4[0], b = p4[1], c = p4[2];
  uint32_t x[12] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z, c.w};
  const int e = w & 3;  // words x[e .. e+8] are needed
  if (e & 2) {
#pragma unroll
    for (int i = 0; i < 10; ++i) x[i] = x[i + 2];
  }
  if (e & 1) {
#pragma unroll
    for (int i = 0; i < 9; ++i) x[i] = x[i + 1];
  }
  const unsigned sh = (unsigned)(j & 1) * 16u;
#pragma unroll
  for (int i = 0; i < 8; ++i) acc[i] += __funnelshift_r(x[i], x[i + 1], sh);
}

template <int G>
__global__ void __launch_bounds__(DD_NT, 2)
    k_dedisp_sb(const uint8_t *__restrict__ s, uint64_t ld, uint64_t ns, uint64_t nch,
                uint64_t dstride, const uint32_t *__restrict__ delays, uint64_t ntrials,
                uint64_t n, float *__restrict__ out, uint64_t ldo, double *__restrict__ part,
                uint64_t ntiles, int cc, int rowcap, int accumulate, unsigned *err,
                long long spin_limit, const SbEntry *__restrict__ plan, uint64_t nsub_total,
                uint64_t sb0, uint64_t block0, int sbstride) {
  static_assert(G <= SB_GMAX, "subband width");
  extern __shared__ __align__(128) uint8_t smem[];
  const size_t bstride = (size_t)cc * rowcap;
  uint16_t *pbuf = reinterpret_cast<uint16_t *>(smem + 2 * bstride);
  __shared__ uint64_t bars[2];
  __shared__ StageInfo info[2];
  __shared__ unsigned long long wsum[DD_NT / 32][SB_TB];
  // the plan entries of each staged chunk's subbands, copied with its rows
  __shared__ __align__(16) SbEntry ents[2][DD_MAXCC / 4];

  const uint64_t t0 = (uint64_t)blockIdx.x * DD_TT;
  const uint64_t d0 = (uint64_t)blockIdx.y * SB_TB;
  const int tl = threadIdx.x;
  const int nchunks = (int)((nch + cc - 1) / cc);
  const SbEntry *pl = plan + (block0 + blockIdx.y) * nsub_total + sb0;

  if (tl == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // Entries of chunk k: subbands [k cc / G, ...) of this block, contiguous in
  // the plan; lane 0 copies them on the chunk's barrier before the rows'
  // copies complete it.
  auto stage_entries = [&](int k, int b) {
    if (tl == 0) {
      const uint64_t e0 = ((uint64_t)k * cc) / G;
      const uint64_t ne = (min((uint64_t)cc, nch - (uint64_t)k * cc) + G - 1) / G;
      const unsigned bytes = (unsigned)(ne * sizeof(SbEntry));
      mbar_expect_tx(&bars[b], bytes);
      bulk_g2s(&ents[b][0], pl + e0, bytes, &bars[b]);
    }
  };
  if (tl < 32) {
    stage_entries(0, 0);
    issue_stage<SB_TB>(s, ld, ns, nch, dstride, delays, ntrials, d0, t0, 0, cc, smem, rowcap,
                       &info[0], &bars[0], 0);
    if (nchunks > 1) {
      stage_entries(1, 1);
      issue_stage<SB_TB>(s, ld, ns, nch, dstride, delays, ntrials, d0, t0, (uint64_t)cc, cc,
                         smem + bstride, rowcap, &info[1], &bars[1], 0);
    }
  }
  uint32_t acc[SB_TB][8];
#pragma unroll
  for (int d = 0; d < SB_TB; ++d)
#pragma unroll
    for (int i = 0; i < 8; ++i) acc[d][i] = 0;

  int failed = -1;
  bool pending = false;  // the pattern buffers hold partials some thread may still read
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
    for (int j0 = 0; j0 < rows; j0 += G) {
      const int gr = min(G, rows - j0);
      const SbEntry &ent = ents[b][j0 / G];
      const int npat = ent.npat;
      if (npat == 0) {
        for (int r = j0; r < j0 + gr; ++r) {
          const uint4 *row16 = reinterpret_cast<const uint4 *>(buf + (size_t)r * rowcap);
#pragma unroll
          for (int d = 0; d < SB_TB; ++d) add_bytes16(row16, info[b].off[r][d] + 16 * tl, acc[d]);
        }
        continue;
      }
      // Stage A: pattern partials over [lo, hi + tile) of the reference delay,
      // once every thread is done reading the previous subband's partials.
      if (pending) __syncthreads();
      for (int p = 0; p < npat; ++p) {
        const int lo = ent.lo[p];
        const int ngr = (DD_TT + (ent.hi[p] - lo) + 15) >> 4;
        uint16_t *dst = pbuf + (size_t)p * sbstride;
        for (int g = tl; g < ngr; g += DD_NT) {
          uint32_t a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
          for (int r = 0; r < gr; ++r) {
            const long long abs0 = (long long)t0 + ent.dref_min + lo + 16 * g + ent.rel[p][r];
            const int off = (int)(abs0 - info[b].base[j0 + r]);
            add_bytes16(reinterpret_cast<const uint4 *>(buf + (size_t)(j0 + r) * rowcap), off, a);
          }
          uint4 *d4 = reinterpret_cast<uint4 *>(dst + 16 * g);
          d4[0] = make_uint4(a[0], a[1], a[2], a[3]);
          d4[1] = make_uint4(a[4], a[5], a[6], a[7]);
        }
      }
      __syncthreads();
      // Stage B: every trial adds its pattern's partial at its shift.
#pragma unroll
      for (int d = 0; d < SB_TB; ++d) {
        const int p = ent.pid[d];
        add_u16x16(pbuf + (size_t)p * sbstride, ent.roff[d] - ent.lo[p] + 16 * tl, acc[d]);
      }
      pending = true;
    }
    __syncthreads();  // every thread is done reading buffer b (rows, entries, partials)
    pending = false;
    if (tl < 32 && k + 2 < nchunks) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      stage_entries(k + 2, b);
      issue_stage<SB_TB>(s, ld, ns, nch, dstride, delays, ntrials, d0, t0,
                         (uint64_t)(k + 2) * cc, cc, smem + b * bstride, rowcap, &info[b],
                         &bars[b], 0);
    }
  }
  if (failed >= 0) {
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
  for (int d = 0; d < SB_TB; ++d) {
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
  if (tl < SB_TB && d0 + tl < ntrials) {
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

// The subband kernel over channel groups (sums of a group stay below 2^16;
// groups start at multiples of G).  PSR_EINVAL (no error recorded) when the
// sample range or the shared memory does not fit this path.
int launch_dedisperse_sb(const DeviceObs &o, const uint32_t *d_delays, uint64_t ntrials,
                         uint64_t n, float *d_out, uint64_t ldo, double *d_part,
                         uint64_t max_spread, unsigned *d_err, cudaStream_t st, long long spin,
                         const SubbandPlan &sb, uint64_t chunk_index) {
  const int G = sb.G;
  const double maxv = o.max_value();
  const uint64_t gch = maxv > 0.0 ? (uint64_t)(65535.0 / maxv) : 0;
  const uint64_t glen = std::min<uint64_t>((gch / G) * G, ((o.nch + G - 1) / G) * G);
  if (glen < (uint64_t)G || (double)o.nch * maxv >= 16777216.0) return PSR_EINVAL;
  const uint64_t ntiles = (n + DD_TT - 1) / DD_TT;
  const int rowcap = (int)(((uint64_t)DD_TT + max_spread + 64 + 15) & ~(uint64_t)15);
  const int sbstride = (int)(((uint64_t)DD_TT + max_spread + 40 + 7) & ~(uint64_t)7);
  int dev = 0;
  PSR_CUDA(cudaGetDevice(&dev));
  int smax = 0, smsm = 0;
  PSR_CUDA(cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  PSR_CUDA(cudaDeviceGetAttribute(&smsm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  const size_t budget = std::min((size_t)smax, (size_t)smsm / 2) - 4096;
  const size_t pbytes = (size_t)SB_PMAX * sbstride * 2;
  if (budget <= pbytes) return PSR_EINVAL;
  int cc = (int)std::min<uint64_t>((uint64_t)DD_MAXCC, (budget - pbytes) / (2 * (size_t)rowcap));
  cc = (cc / G) * G;
  if (cc < G) return PSR_EINVAL;
  const size_t smem = 2 * (size_t)cc * rowcap + pbytes;
  const SbEntry *plan = sb.entries.as<SbEntry>();
  auto kern = G == 4 ? k_dedisp_sb<4> : k_dedisp_sb<8>;
  if (G != 4 && G != 8) return PSR_EINVAL;
  PSR_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((unsigned)ntiles, (unsigned)((ntrials + SB_TB - 1) / SB_TB));
  for (uint64_t c0 = 0; c0 < o.nch; c0 += glen) {
    const uint64_t ng = std::min(glen, o.nch - c0);
    const int ccg = (int)std::min<uint64_t>((uint64_t)cc, ((ng + G - 1) / G) * G);
    kern<<<grid, DD_NT, smem, st>>>(o.samples.as<uint8_t>() + c0 * o.ld, o.ld, o.ns, ng, o.nch,
                                    d_delays + c0, ntrials, n, d_out, ldo, d_part, ntiles, ccg,
                                    rowcap, c0 > 0 ? 1 : 0, d_err, spin, plan, sb.nsub, c0 / G,
                                    sb.block0[chunk_index], sbstride);
    PSR_CUDA(cudaGetLastError());
  }
  return PSR_OK;
}

namespace {
std::atomic<int> g_subbands{-1};
}
int dedisp_subbands_default(const DeviceObs &o) {
  const int g = g_subbands.load();
  if (g >= 0) return g;
  // Measured on a GB300 with the word-cache channel-by-channel kernel: the
  // whole 8000-trial survey search (4096 x 8-bit channels, 2^23 samples)
  // takes 13.39 s with subbands of 8 and 14.13 s channel by channel; at
  // 64-1024 8-bit channels subbands cost about 8%, and on <= 4-bit samples
  // the byte-lane kernel is faster.  Batches tune it per shape class.
  return o.kind == SAMPLE_U8 && o.h.nbits == 8 && o.nch >= 2048 ? 8 : 0;
}

// Cost of one (block, subband) in thread instructions per 16 samples, for
// the choice between stage A/B and direct adds: a shifted 16-byte add is
// about 33, a shifted 16-sample u16 add about 37, plus two barriers.
bool subband_pays(int npat, int ge, int tbe) {
  return npat * ge * 33 + tbe * 37 + 40 < tbe * ge * 33;
}

int build_subband_plan(const std::vector<uint32_t> &tab, uint64_t nch,
                       const std::vector<uint64_t> &cstart, int G, SubbandPlan &plan,
                       cudaStream_t st) {
  plan.G = 0;
  plan.nsub = 0;
  plan.block0.clear();
  plan.reused = plan.direct = 0;
  if ((G != 4 && G != 8) || cstart.size() < 2) return PSR_OK;
  const uint64_t nsub = (nch + G - 1) / G;
  std::vector<uint64_t> block0;
  uint64_t nblocks = 0;
  for (size_t ci = 0; ci + 1 < cstart.size(); ++ci) {
    block0.push_back(nblocks);
    nblocks += (cstart[ci + 1] - cstart[ci] + SB_TB - 1) / SB_TB;
  }
  std::vector<SbEntry> ent(nblocks * nsub);
  uint64_t nsb = 0, ndirect = 0;
  for (size_t ci = 0; ci + 1 < cstart.size(); ++ci) {
    const uint64_t ta = cstart[ci], tz = cstart[ci + 1];
    for (uint64_t b = 0; ta + b * SB_TB < tz; ++b) {
      const uint64_t tb0 = ta + b * SB_TB;
      const int tbe = (int)std::min<uint64_t>(SB_TB, tz - tb0);
      for (uint64_t j = 0; j < nsub; ++j) {
        SbEntry e{};
        const uint64_t ca = j * G;
        const int ge = (int)std::min<uint64_t>(G, nch - ca);
        uint32_t dref[SB_TB];
        int32_t dmin = INT32_MAX, dmaxr = 0;
        for (int d = 0; d < SB_TB; ++d) {
          // trials past the chunk repeat its last trial, as the kernel's staging does
          const uint64_t tr = tb0 + (uint64_t)std::min(d, tbe - 1);
          uint32_t m = 0xffffffffu;
          for (int c = 0; c < ge; ++c) m = std::min(m, tab[tr * nch + ca + c]);
          dref[d] = m;
          dmin = std::min(dmin, (int32_t)m);
          dmaxr = std::max(dmaxr, (int32_t)m);
        }
        bool ok = dmaxr - dmin < 65536;
        int npat = 0;
        for (int d = 0; d < SB_TB && ok; ++d) {
          const uint64_t tr = tb0 + (uint64_t)std::min(d, tbe - 1);
          uint16_t rel[SB_GMAX] = {0};
          for (int c = 0; c < ge; ++c) {
            const uint32_t r = tab[tr * nch + ca + c] - dref[d];
            if (r > 65535u) ok = false;
            rel[c] = (uint16_t)r;
          }
          int p = 0;
          while (p < npat && std::memcmp(e.rel[p], rel, sizeof(rel)) != 0) ++p;
          if (p == npat) {
            if (npat == SB_PMAX) {
              ok = false;
              break;
            }
            std::memcpy(e.rel[p], rel, sizeof(rel));
            e.lo[p] = 0xffff;
            e.hi[p] = 0;
            ++npat;
          }
          const uint16_t ro = (uint16_t)(dref[d] - (uint32_t)dmin);
          e.pid[d] = (uint8_t)p;
          e.roff[d] = ro;
          e.lo[p] = std::min(e.lo[p], ro);
          e.hi[p] = std::max(e.hi[p], ro);
        }
        if (ok && subband_pays(npat, ge, tbe)) {
          e.npat = (uint8_t)npat;
          e.dref_min = dmin;
          ++nsb;
        } else {
          e = SbEntry{};
          ++ndirect;
        }
        ent[(block0[ci] + b) * nsub + j] = e;
      }
    }
  }
  PSR_TRY(plan.entries.ensure(ent.size() * sizeof(SbEntry)));
  PSR_CUDA(cudaMemcpyAsync(plan.entries.p, ent.data(), ent.size() * sizeof(SbEntry),
                           cudaMemcpyHostToDevice, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  plan.G = G;
  plan.nsub = nsub;
  plan.block0 = block0;
  plan.reused = nsb;
  plan.direct = ndirect;
  return PSR_OK;
}

int launch_dedisperse_ex(const DeviceObs &o, const uint32_t *d_delays, uint64_t ntrials,
                         uint64_t n, float *d_out, uint64_t ldo, double *d_part,
                         double *d_sums, float *d_means, uint64_t max_spread, unsigned *d_err,
                         cudaStream_t st, long long spin_limit, int arm_only, bool want_means,
                         const SubbandPlan *sb, uint64_t chunk_index) {
  const long long spin = spin_limit > 0 ? spin_limit : DD_SPIN_LIMIT;
  if (sb && sb->G && !arm_only && o.kind == SAMPLE_U8 && chunk_index < sb->block0.size()) {
    int rc = launch_dedisperse_sb(o, d_delays, ntrials, n, d_out, ldo, d_part, max_spread,
                                  d_err, st, spin, *sb, chunk_index);
    if (rc == PSR_OK) {
      if (want_means) {
        const uint64_t ntiles = (n + DD_TT - 1) / DD_TT;
        k_reduce_parts<<<(unsigned)((ntrials + 127) / 128), 128, 0, st>>>(
            d_part, ntiles, ntrials, n, d_sums, d_means, d_out, ldo, 0);
        PSR_CUDA(cudaGetLastError());
      }
      return PSR_OK;
    }
    if (rc != PSR_EINVAL) return rc;  // EINVAL: this shape does not fit; take the kernels below
  }
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
    // The CTA's delay block ([trials per CTA][channels of the group], u32) is
    // preloaded into shared memory when it takes at most 16 KB.
    const int group = (int)(255.0 / maxv);
    const size_t dly_bytes = (size_t)(group >= 2 ? DD_DB8 : DD_DB) * glen * 4;
    const int preload = dly_bytes <= 16384 && dly_bytes + 2 * (size_t)rowcap <= budget;
    if (preload) budget -= dly_bytes;
    int cc = (int)std::min<uint64_t>({(uint64_t)DD_MAXCC, glen, budget / (2 * (size_t)rowcap)});
    if (cc >= 1) {
      size_t smem = 2 * (size_t)cc * rowcap + (preload ? dly_bytes : 0);
      for (uint64_t c0 = 0; c0 < o.nch; c0 += glen) {
        const uint64_t ng = std::min(glen, o.nch - c0);
        const uint8_t *sg = o.samples.as<uint8_t>() + c0 * o.ld;
        const uint32_t *dg = d_delays + c0;
        const int acc = c0 > 0 ? 1 : 0;
        const int ccg = (int)std::min<uint64_t>((uint64_t)cc, ng);
        auto run = [&](auto kern, int db, int grp) -> int {
          dim3 grid((unsigned)ntiles, (unsigned)((ntrials + db - 1) / db));
          PSR_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
          kern<<<grid, DD_NT, smem, st>>>(sg, o.ld, o.ns, ng, o.nch, dg, ntrials, n, d_out, ldo,
                                          d_part, ntiles, ccg, rowcap, grp, acc, d_err, spin,
                                          arm_only);
          return PSR_OK;
        };
        int rc;
        if (group >= 2)
          rc = preload ? run(k_dedisp_u8<true, DD_DB8, true>, DD_DB8, group)
                       : run(k_dedisp_u8<true, DD_DB8, false>, DD_DB8, group);
        else
          rc = preload ? run(k_dedisp_u8<false, DD_DB, true>, DD_DB, 1)
                       : run(k_dedisp_u8<false, DD_DB, false>, DD_DB, 1);
        if (rc != PSR_OK) return rc;
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

extern "C" int psr_set_dedisp_subbands(int subbands) {
  if (subbands != -1 && subbands != 0 && subbands != 4 && subbands != 8) {
    psr::set_error("set_dedisp_subbands: -1, 0, 4 or 8");
    return PSR_EINVAL;
  }
  psr::g_subbands.store(subbands);
  return PSR_OK;
}
