// K4 real FFT + raw power (search/src/lib.rs:35-44).
//
// The FFT is a fixed FP32 algorithm, reproduced operation for operation by
// the CPU oracle so that spectra (and everything downstream) are bit-exact:
//   N = 2*next_pow2(len) real points, M = N/2 complex points,
//   z[n] = x[2n] + i x[2n+1],  x[i] = series[i] - (f32)mean  (0 beyond len).
//   Twiddles W_N^x come from a quarter table ((f32)cos, (f32)sin of 2 pi r/N
//   for r <= N/8, mirrored above) and exact quadrant symmetry.
//   cmul(a, w) = (fma(a.re, w.re, -(a.im*w.im)), fma(a.re, w.im, a.im*w.re)).
//   M <= 4096: one Stockham sub-FFT.  Otherwise four-step M = M1*M2,
//   M1 = 2^ceil(m/2): pass 1 = column sub-FFTs over n1 (n = n1*M2 + n2) and
//   the twiddle W_M^(n2*k1); pass 2 = row sub-FFTs, fused with the real
//   post-processing X[k] = 0.5*(e.re + t.im, e.im - t.re), e = a + b,
//   t = cmul(a - b, W_N^k), a = Z[k], b = conj(Z[M-k]), and |X|^2.
//   Sub-FFT of size L: Stockham autosort stages with radices
//   [16]*(q/4) + [2|4|8]; DFT_8 = 2x4 and DFT_16 = 4x4 four-step with the
//   internal twiddles W_R^(n2*k1).
// A CTA transforms C columns held in shared memory position-major with one
// padding slot every 16 (free of bank conflicts for the row-wise global
// loads, every Stockham access and the drains).  Every size is a template parameter, so all index
// arithmetic reduces to shifts and masks; each thread owns exactly one
// radix-16 butterfly per stage.  Stages are in place: every thread loads its
// inputs, the block synchronises, then stores.
#include <cuda_runtime.h>

#include <type_traits>

#include <algorithm>
#include <cmath>
#include <vector>

#include "psr_internal.h"

namespace psr {
namespace {

constexpr int LB = 8;  // global loads in flight per thread when staging a tile

__host__ __device__ constexpr int ilog2(int x) { return x <= 1 ? 0 : 1 + ilog2(x >> 1); }
__host__ __device__ constexpr int cols_for(int L) {
  return L >= 8192 ? 1 : (8192 / L > 16 ? 16 : 8192 / L);
}
__host__ __device__ constexpr int threads_for(int L, int C) {
  return ((L / 16) * C < 32 ? 32 : (L / 16) * C);
}

// Shared-memory slot of (position, column) for C columns: the linear index
// e = pos*C + col padded by one slot every 16 (conflict-free for the fill,
// every Stockham load/store pattern and the drains of both passes).
template <int C>
__device__ __forceinline__ int lay(int pos, int col) {
  const int e = pos * C + col;
  return e + (e >> 4);
}
template <int L, int C>
__host__ __device__ constexpr int lay_slots() {
  return L * C + (L * C) / 16 + 1;
}

__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  return make_float2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y));
}
__device__ __forceinline__ float2 cmul(float2 a, float2 w) {
  return make_float2(__fmaf_rn(a.x, w.x, -__fmul_rn(a.y, w.y)),
                     __fmaf_rn(a.x, w.y, __fmul_rn(a.y, w.x)));
}
__device__ __forceinline__ float2 mul_mi(float2 d) { return make_float2(d.y, -d.x); }

// W_N^x for x in [0, N) from the quarter table (lq = log2(N/4)).
// 8-byte asynchronous global -> shared copy (no registers held while in flight).
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

__device__ __forceinline__ float2 twN(const float2 *__restrict__ Q, uint32_t x, int lq) {
  const uint32_t q = x >> lq, r = x & ((1u << lq) - 1u);
  const float2 v = __ldg(&Q[r]);
  switch (q & 3u) {
    case 0: return make_float2(v.x, -v.y);
    case 1: return make_float2(-v.y, -v.x);
    case 2: return make_float2(-v.x, v.y);
    default: return make_float2(v.y, v.x);
  }
}

__device__ __forceinline__ void dft2(float2 &v0, float2 &v1) {
  const float2 a = v0, b = v1;
  v0 = cadd(a, b);
  v1 = csub(a, b);
}
__device__ __forceinline__ void dft4(float2 &v0, float2 &v1, float2 &v2, float2 &v3) {
  float2 a = cadd(v0, v2), b = csub(v0, v2);
  float2 c = cadd(v1, v3), d = mul_mi(csub(v1, v3));
  v0 = cadd(a, c);
  v1 = cadd(b, d);
  v2 = csub(a, c);
  v3 = csub(b, d);
}
// The internal twiddles of the radix-8 and radix-16 butterflies, W_16^y for
// y in {1, 2, 3, 4, 6, 9}, held in registers.  W_L^(y L/16) is the table
// entry for x = y N/16 whatever L is, so one set serves every sub-FFT size;
// load_w16 reads them from a sub-FFT's table (values identical to the table
// lookups they replace).
struct W16 {
  float2 w1, w2, w3, w4, w6, w9;
  template <int Y>
  __device__ __forceinline__ float2 get() const {
    static_assert(Y == 1 || Y == 2 || Y == 3 || Y == 4 || Y == 6 || Y == 9, "W_16 power");
    if constexpr (Y == 1) return w1;
    else if constexpr (Y == 2) return w2;
    else if constexpr (Y == 3) return w3;
    else if constexpr (Y == 4) return w4;
    else if constexpr (Y == 6) return w6;
    else return w9;
  }
};
template <int L>
__device__ __forceinline__ W16 load_w16(const float2 *Wl) {
  W16 c{};
  if constexpr (L >= 16) {
    c.w1 = Wl[1 * (L / 16)];
    c.w2 = Wl[2 * (L / 16)];
    c.w3 = Wl[3 * (L / 16)];
    c.w4 = Wl[4 * (L / 16)];
    c.w6 = Wl[6 * (L / 16)];
    c.w9 = Wl[9 * (L / 16)];
  } else if constexpr (L == 8) {  // W_8^n2 = W_16^(2 n2)
    c.w2 = Wl[1];
    c.w4 = Wl[2];
    c.w6 = Wl[3];
  }
  return c;
}

// W_R^y = W_16^(y 16/R).
__device__ __forceinline__ void dft8(float2 *v, const W16 &c) {
  float2 u[4][2];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    float2 a = v[n2], b = v[n2 + 4];
    dft2(a, b);
    u[n2][0] = a;
    u[n2][1] = b;
  }
  u[1][1] = cmul(u[1][1], c.get<2>());
  u[2][1] = cmul(u[2][1], c.get<4>());
  u[3][1] = cmul(u[3][1], c.get<6>());
#pragma unroll
  for (int k1 = 0; k1 < 2; ++k1) {
    float2 a = u[0][k1], b = u[1][k1], c = u[2][k1], d = u[3][k1];
    dft4(a, b, c, d);
    v[k1] = a;
    v[k1 + 2] = b;
    v[k1 + 4] = c;
    v[k1 + 6] = d;
  }
}
__device__ __forceinline__ void dft16(float2 *v, const W16 &c) {
  float2 u[4][4];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    float2 a = v[n2], b = v[n2 + 4], c = v[n2 + 8], d = v[n2 + 12];
    dft4(a, b, c, d);
    u[n2][0] = a;
    u[n2][1] = b;
    u[n2][2] = c;
    u[n2][3] = d;
  }
  u[1][1] = cmul(u[1][1], c.get<1>());
  u[1][2] = cmul(u[1][2], c.get<2>());
  u[1][3] = cmul(u[1][3], c.get<3>());
  u[2][1] = cmul(u[2][1], c.get<2>());
  u[2][2] = cmul(u[2][2], c.get<4>());
  u[2][3] = cmul(u[2][3], c.get<6>());
  u[3][1] = cmul(u[3][1], c.get<3>());
  u[3][2] = cmul(u[3][2], c.get<6>());
  u[3][3] = cmul(u[3][3], c.get<9>());
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    float2 a = u[0][k1], b = u[1][k1], c = u[2][k1], d = u[3][k1];
    dft4(a, b, c, d);
    v[k1] = a;
    v[k1 + 4] = b;
    v[k1 + 8] = c;
    v[k1 + 12] = d;
  }
}

template <int R>
__device__ __forceinline__ void dftR(float2 *v, const W16 &c) {
  if constexpr (R == 2) dft2(v[0], v[1]);
  else if constexpr (R == 4) dft4(v[0], v[1], v[2], v[3]);
  else if constexpr (R == 8) dft8(v, c);
  else dft16(v, c);
}

// One in-place Stockham stage (radix R, Ns = product of earlier radices) on
// C columns of length L; NT threads, each owning 16/R butterflies.
// Slot distance of D positions when D*C is a multiple of 16 (the padding is
// then D*C/16 slots): lay<C>(p + D, c) = lay<C>(p, c) + lay_step<C, D>().
template <int C, int D>
__host__ __device__ constexpr int lay_step() {
  return D * C + (D * C) / 16;
}

template <int R, int L, int C, int NT, int Ns>
__device__ __forceinline__ void stage(float2 *sm, const float2 *Wl, const W16 &c16) {
  constexpr int nb = L / R;
  constexpr int total = nb * C;
  constexpr int BPT = (total + NT - 1) / NT;
  float2 v[BPT][R];
#pragma unroll
  for (int i = 0; i < BPT; ++i) {
    const int w = (int)threadIdx.x + i * NT;
    if (total % NT == 0 || w < total) {
      const int col = w % C, j = w / C;
      if constexpr ((nb * C) % 16 == 0) {
        const float2 *src = sm + lay<C>(j, col);
#pragma unroll
        for (int r = 0; r < R; ++r) v[i][r] = src[r * lay_step<C, nb>()];
      } else {
#pragma unroll
        for (int r = 0; r < R; ++r) v[i][r] = sm[lay<C>(j + r * nb, col)];
      }
      if constexpr (Ns > 1) {
        const int k = j % Ns;
        if (k != 0) {
#pragma unroll
          for (int r = 1; r < R; ++r) v[i][r] = cmul(v[i][r], Wl[r * k * (L / (Ns * R))]);
        }
      }
      dftR<R>(v[i], c16);
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < BPT; ++i) {
    const int w = (int)threadIdx.x + i * NT;
    if (total % NT == 0 || w < total) {
      const int col = w % C, j = w / C;
      const int base = (j / Ns) * Ns * R + j % Ns;
      if constexpr ((Ns * C) % 16 == 0) {
        float2 *dst = sm + lay<C>(base, col);
#pragma unroll
        for (int r = 0; r < R; ++r) dst[r * lay_step<C, Ns>()] = v[i][r];
      } else {
#pragma unroll
        for (int r = 0; r < R; ++r) sm[lay<C>(base + r * Ns, col)] = v[i][r];
      }
    }
  }
  __syncthreads();
}

template <int L, int C, int NT, int s>
__device__ __forceinline__ void stages16(float2 *sm, const float2 *Wl, const W16 &c) {
  if constexpr (s < ilog2(L) / 4) {
    stage<16, L, C, NT, (1 << (4 * s))>(sm, Wl, c);
    stages16<L, C, NT, s + 1>(sm, Wl, c);
  }
}

// The stages after the first radix-16 stage (used when stage 0 runs fused
// with the global loads).
template <int L, int C, int NT>
__device__ __forceinline__ void subfft_rest(float2 *sm, const float2 *Wl, const W16 &c) {
  constexpr int q = ilog2(L);
  constexpr int NsLast = 1 << (4 * (q / 4));
  stages16<L, C, NT, 1>(sm, Wl, c);
  if constexpr (q % 4 == 1) stage<2, L, C, NT, NsLast>(sm, Wl, c);
  else if constexpr (q % 4 == 2) stage<4, L, C, NT, NsLast>(sm, Wl, c);
  else if constexpr (q % 4 == 3) stage<8, L, C, NT, NsLast>(sm, Wl, c);
}

template <int L, int C, int NT>
__device__ __forceinline__ void subfft(float2 *sm, const float2 *Wl, const W16 &c) {
  constexpr int q = ilog2(L);
  constexpr int NsLast = 1 << (4 * (q / 4));
  stages16<L, C, NT, 0>(sm, Wl, c);
  if constexpr (q % 4 == 1) stage<2, L, C, NT, NsLast>(sm, Wl, c);
  else if constexpr (q % 4 == 2) stage<4, L, C, NT, NsLast>(sm, Wl, c);
  else if constexpr (q % 4 == 3) stage<8, L, C, NT, NsLast>(sm, Wl, c);
}

template <int L>
__device__ __forceinline__ void build_wl(float2 *Wl, uint32_t N, const float2 *Q, int lq) {
  const uint32_t stride = N / (uint32_t)L;
  for (int y = threadIdx.x; y < L; y += blockDim.x) Wl[y] = twN(Q, (uint32_t)y * stride, lq);
}

// Real post-processing of one bin: a = Z[k], b = conj(Z[M-k]).
__device__ __forceinline__ float post_power(float2 a, float2 zb, float2 w) {
  const float2 b = make_float2(zb.x, -zb.y);
  const float2 e = cadd(a, b), o = csub(a, b);
  const float2 t = cmul(o, w);
  const float xr = __fmul_rn(0.5f, __fadd_rn(e.x, t.y));
  const float xi = __fmul_rn(0.5f, __fsub_rn(e.y, t.x));
  return __fadd_rn(__fmul_rn(xr, xr), __fmul_rn(xi, xi));
}

// Both bins of a mirrored pair at once: pk from a = zk, b = conj(zm) with
// W_N^k = w, and pm from a = zm, b = conj(zk) with W_N^(M-k) = (-w.re, w.im).
// The mirror's e, o and t are exactly (e.re, -e.im), (-o.re, o.im) and
// (t.re, -t.im) (round to nearest is symmetric in sign and the fma products
// are the same), so pm equals post_power(zm, zk, (-w.re, w.im)) bit for bit.
__device__ __forceinline__ void post_power_pair(float2 zk, float2 zm, float2 w, float &pk,
                                                float &pm) {
  const float2 b = make_float2(zm.x, -zm.y);
  const float2 e = cadd(zk, b), o = csub(zk, b);
  const float2 t = cmul(o, w);
  const float xr = __fmul_rn(0.5f, __fadd_rn(e.x, t.y));
  const float xi = __fmul_rn(0.5f, __fsub_rn(e.y, t.x));
  pk = __fadd_rn(__fmul_rn(xr, xr), __fmul_rn(xi, xi));
  const float yr = __fmul_rn(0.5f, __fsub_rn(e.x, t.y));
  const float yi = __fmul_rn(0.5f, __fadd_rn(e.y, t.x));  // -(mirror's xi)
  pm = __fadd_rn(__fmul_rn(yr, yr), __fmul_rn(yi, yi));
}

__device__ __forceinline__ float2 load_z(const float *__restrict__ row, uint64_t len, uint64_t n,
                                         float mean) {
  const uint64_t i0 = 2 * n;
  float x0 = 0.0f, x1 = 0.0f;
  if (i0 + 1 < len) {
    const float2 p = *reinterpret_cast<const float2 *>(row + i0);
    x0 = __fsub_rn(p.x, mean);
    x1 = __fsub_rn(p.y, mean);
  } else if (i0 < len) {
    x0 = __fsub_rn(row[i0], mean);
  }
  return make_float2(x0, x1);
}

// Partial sums of the power spectrum for the normalisation floor: f32
// TwoSum (error-free transformation) per thread, f64 across threads.
struct Acc2 {
  float hi = 0.0f, lo = 0.0f;
  __device__ __forceinline__ void add(float b) {
    const float s = __fadd_rn(hi, b);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    hi = s;
    lo = __fadd_rn(lo, err);
  }
};

// Block total of the per-thread (hi, lo) pairs: TwoSum merges across the
// warp in f32, f64 only for the final per-warp pairs (thread 0).
template <int NT>
__device__ __forceinline__ void block_sum_store(Acc2 acc, double *dst) {
  __shared__ float2 red[NT / 32 > 0 ? NT / 32 : 1];
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const float oh = __shfl_down_sync(0xffffffffu, acc.hi, o);
    const float ol = __shfl_down_sync(0xffffffffu, acc.lo, o);
    acc.add(oh);
    acc.lo = __fadd_rn(acc.lo, ol);
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_float2(acc.hi, acc.lo);
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) t += (double)red[w].x + (double)red[w].y;
    *dst = t;
  }
}

// Whole transform in one CTA per trial (M <= 4096).
template <int M>
__global__ void __launch_bounds__(threads_for(M, 1))
    k_fft_small(const float *__restrict__ series, uint64_t lds, uint64_t len,
                const float *__restrict__ means, const float2 *__restrict__ Q, int lq,
                uint32_t N, float *__restrict__ power, uint64_t ldp,
                double *__restrict__ psum) {
  constexpr int NT = threads_for(M, 1);
  extern __shared__ float2 dyn[];
  float2 *Wl = dyn;      // M entries
  float2 *sm = dyn + M;  // lay_slots<M, 1>() entries
  const uint64_t trial = blockIdx.x;
  const float *row = series + trial * lds;
  const float mean = means[trial];
  build_wl<M>(Wl, N, Q, lq);
  for (int n = threadIdx.x; n < M; n += NT) sm[lay<1>(n, 0)] = load_z(row, len, (uint64_t)n, mean);
  __syncthreads();
  const W16 c16 = load_w16<M>(Wl);
  subfft<M, 1, NT>(sm, Wl, c16);
  Acc2 acc;
  float *out = power + trial * ldp;
  for (int k = threadIdx.x; k <= M; k += NT) {
    const float p =
        post_power(sm[lay<1>(k % M, 0)], sm[lay<1>((M - k) % M, 0)], twN(Q, (uint32_t)k, lq));
    out[k] = p;
    acc.add(p);
  }
  block_sum_store<NT>(acc, psum + trial);
}

// z[n] from a staged pair of series values (as load_z reads them).
__device__ __forceinline__ float2 staged_z(float2 p, uint64_t len, uint64_t n, float mean) {
  const uint64_t i0 = 2 * n;
  if (i0 + 1 < len) return make_float2(__fsub_rn(p.x, mean), __fsub_rn(p.y, mean));
  if (i0 < len) return make_float2(__fsub_rn(p.x, mean), 0.0f);
  return make_float2(0.0f, 0.0f);
}

// 16-byte asynchronous global -> shared copy, cached in L2 only.
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src)
               : "memory");
}

// Copies the non-zero rows n1 < ceil(nz / M2) of column group n2_0 of `row`
// into stg[n1 * C + c] (float pairs), 16 bytes per thread and step; chunks
// starting at or past len are left alone (stage 0 never reads them).
template <int M1, int M2>
__device__ __forceinline__ void p1_stage_rows(float2 *stg, const float *__restrict__ row,
                                              uint64_t len, uint32_t n2_0) {
  constexpr int C = cols_for(M1), NT = threads_for(M1, C);
  static_assert(C % 2 == 0, "16-byte chunks of complex pairs");
  const uint64_t nz = (len + 1) / 2;
  const int rows = (int)((nz + M2 - 1) / M2);
  const int nchunk = rows * (C / 2);
  for (int q = threadIdx.x; q < nchunk; q += NT) {
    const int n1 = q / (C / 2), part = q % (C / 2);
    const uint64_t f = 2 * ((uint64_t)n1 * M2 + n2_0) + 4 * (uint64_t)part;
    if (f < len) cp_async16(stg + n1 * C + 2 * part, row + f);
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
}

// Pass 1 on one column group: C columns n2 in [n2_0, n2_0 + C) of trial
// `row` (length M1 over n1), then W_M^(n2*k1), written to out[k1*M2 + n2].
// stg (if not null) holds the group's non-zero rows (p1_stage_rows);
// after_stage0() runs once every thread is done with stg.
template <int M1, int M2, class Hook>
__device__ __forceinline__ void p1_group(float2 *sm, const float2 *Wl, const W16 &c16,
                                         const float *__restrict__ row, uint64_t len,
                                         float mean, uint32_t n2_0,
                                         const float2 *__restrict__ tw1,
                                         float2 *__restrict__ out, const float2 *stg,
                                         Hook after_stage0) {
  constexpr int C = cols_for(M1), NT = threads_for(M1, C);
  constexpr int total = M1 * C;
  const uint64_t nz = (len + 1) / 2;  // complex inputs that can be non-zero
  {
    // Stage 0 (radix 16, Ns = 1) straight from global memory (or the staged
    // rows): butterfly (col, j) takes positions j + r*M1/16 of its column and
    // stores its outputs at 16j + r.  The zero padding (n >= nz) is never
    // loaded.
    constexpr int nb = M1 / 16;
    constexpr int nbt = nb * C;
    constexpr int BPT = (nbt + NT - 1) / NT;
#pragma unroll
    for (int i = 0; i < BPT; ++i) {
      const int w = (int)threadIdx.x + i * NT;
      if (nbt % NT == 0 || w < nbt) {
        const int col = w % C, j = w / C;
        float2 v[16];
        if (stg) {
#pragma unroll
          for (int r = 0; r < 16; ++r) {
            const uint64_t n = (uint64_t)(j + r * nb) * M2 + n2_0 + col;
            v[r] = n < nz ? staged_z(stg[(j + r * nb) * C + col], len, n, mean)
                          : make_float2(0.0f, 0.0f);
          }
        } else {
#pragma unroll
          for (int r = 0; r < 16; ++r) {
            const uint64_t n = (uint64_t)(j + r * nb) * M2 + n2_0 + col;
            v[r] = n < nz ? load_z(row, len, n, mean) : make_float2(0.0f, 0.0f);
          }
        }
        dft16(v, c16);
        if constexpr (16 % C == 0) {
          // e = (16j + r) C + col with col < C | 16: the padding of r C +
          // col is (r C) / 16, so every r is a constant offset
          float2 *dst = sm + 17 * C * j + col;
#pragma unroll
          for (int r = 0; r < 16; ++r) dst[r * C + (r * C) / 16] = v[r];
        } else {
#pragma unroll
          for (int r = 0; r < 16; ++r) sm[lay<C>(16 * j + r, col)] = v[r];
        }
      }
    }
  }
  __syncthreads();
  after_stage0();
  subfft_rest<M1, C, NT>(sm, Wl, c16);
  // W_M^(n2*k1) comes from a table laid out like the output, Tw1[k1*M2 +
  // n2] (values identical to the quarter-table lookup): reads coalesce.
  if constexpr (NT % C == 0 && 16 % C == 0) {
    // thread t drains column t % C at rows k1 = t / C + i NT / C: slot
    // lay<C>(k1, col) = C k1 + col + (C k1) / 16 advances by a constant
    constexpr int KS = NT / C;  // row step
    const int col = (int)threadIdx.x % C, k10 = (int)threadIdx.x / C;
    const uint32_t n2 = n2_0 + (uint32_t)col;
    const float2 *src = sm + C * k10 + col + (C * k10) / 16;
    const float2 *tws = tw1 + (uint64_t)k10 * M2 + n2;
    float2 *dst = out + (uint64_t)k10 * M2 + n2;
    constexpr int NI = M1 / KS;
#pragma unroll 1
    for (int i0 = 0; i0 < NI; i0 += LB) {
      float2 w[LB];
#pragma unroll
      for (int u = 0; u < LB; ++u)
        w[u] = i0 + u < NI ? __ldg(tws + (uint64_t)(i0 + u) * KS * M2)
                           : make_float2(1.0f, 0.0f);
#pragma unroll
      for (int u = 0; u < LB; ++u) {
        if (i0 + u < NI) {
          const int k1 = k10 + (i0 + u) * KS;
          float2 v = src[(i0 + u) * lay_step<C, KS>()];
          if (n2 * (uint32_t)k1 != 0) v = cmul(v, w[u]);
          dst[(uint64_t)(i0 + u) * KS * M2] = v;
        }
      }
    }
  } else {
#pragma unroll 1
    for (int base = 0; base < total; base += LB * NT) {
      float2 w[LB];
#pragma unroll
      for (int u = 0; u < LB; ++u) {
        const int idx = base + u * NT + (int)threadIdx.x;
        w[u] = idx < total ? __ldg(&tw1[(uint64_t)(idx / C) * M2 + n2_0 + (idx % C)])
                           : make_float2(1.0f, 0.0f);
      }
#pragma unroll
      for (int u = 0; u < LB; ++u) {
        const int idx = base + u * NT + (int)threadIdx.x;
        if (idx < total) {
          const int col = idx % C, k1 = idx / C;
          const uint32_t n2 = n2_0 + (uint32_t)col;
          float2 v = sm[lay<C>(k1, col)];
          if (n2 * (uint32_t)k1 != 0) v = cmul(v, w[u]);
          out[(uint64_t)k1 * M2 + n2] = v;
        }
      }
    }
  }
}

// Pass 1: column groups of every trial, persistent: CTA b takes groups b,
// b + gridDim.x, ... (group g = trial g / (M2/C), columns (g % (M2/C)) C
// ...), builds the twiddle table once, and while it transforms one group
// prefetches the next group's samples into L2 (one 64-byte run of C complex
// inputs per row).
// STAGED: the next group's non-zero rows are copied into shared memory
// (cp.async) while the CTA transforms the current group, instead of
// prefetched into L2, so stage 0 reads shared memory.
template <int M1, int M2, bool STAGED>
__global__ void __launch_bounds__(threads_for(M1, cols_for(M1)), 2)
    k_fft_pass1(const float *__restrict__ series, uint64_t lds, uint64_t len,
                const float *__restrict__ means, const float2 *__restrict__ Q, int lq,
                uint32_t N, const float2 *__restrict__ tw1, float2 *__restrict__ work,
                uint32_t ngroups) {
  constexpr int C = cols_for(M1);
  constexpr uint32_t M = (uint32_t)M1 * M2;
  constexpr uint32_t GPT = M2 / C;  // column groups per trial
  extern __shared__ float2 dyn[];
  float2 *Wl = dyn;       // M1 entries
  float2 *sm = dyn + M1;  // lay_slots<M1, C>() entries
  // staged rows after sm, rounded up to 16 bytes (the launch adds one slot)
  float2 *stg = STAGED ? reinterpret_cast<float2 *>(
                             (reinterpret_cast<uintptr_t>(sm + lay_slots<M1, C>()) + 15) &
                             ~(uintptr_t)15)
                       : nullptr;
  if constexpr (STAGED) {
    if (blockIdx.x < ngroups)
      p1_stage_rows<M1, M2>(stg, series + (uint64_t)(blockIdx.x / GPT) * lds, len,
                            (blockIdx.x % GPT) * (uint32_t)C);
  }
  build_wl<M1>(Wl, N, Q, lq);
  const uint64_t nz = (len + 1) / 2;
  __syncthreads();  // Wl
  const W16 c16 = load_w16<M1>(Wl);
  for (uint32_t grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
    const uint64_t trial = grp / GPT;
    const uint32_t n2_0 = (grp % GPT) * (uint32_t)C;
    const uint32_t nx = grp + gridDim.x;
    if constexpr (STAGED) {
      asm volatile("cp.async.wait_all;" ::: "memory");
      __syncthreads();  // this group's rows are in stg
      p1_group<M1, M2>(sm, Wl, c16, series + trial * lds, len, means[trial], n2_0, tw1,
                       work + trial * (uint64_t)M, stg, [&]() {
                         if (nx < ngroups)
                           p1_stage_rows<M1, M2>(stg, series + (uint64_t)(nx / GPT) * lds, len,
                                                 (nx % GPT) * (uint32_t)C);
                       });
    } else {
      // (only inputs the next group loads: complex index < nz)
      const uint64_t pn = (uint64_t)threadIdx.x * M2 + (nx % GPT) * (uint32_t)C;
      if (nx < ngroups && pn < nz) {
        const float *pr = series + (uint64_t)(nx / GPT) * lds + 2 * pn;
        asm volatile("prefetch.global.L2 [%0];" ::"l"(pr));
      }
      p1_group<M1, M2>(sm, Wl, c16, series + trial * lds, len, means[trial], n2_0, tw1,
                       work + trial * (uint64_t)M, nullptr, []() {});
    }
    __syncthreads();  // the next group's stage 0 overwrites sm
  }
}

// Pass 2 on one row group of one trial: the row sub-FFTs of length M2, then
// the real post-processing and |X|^2.  Group 0 holds rows 0 and M1/2; group
// g >= 1 holds rows kb..kb+h-1 (kb = 1 + (g-1)*H) and M1-kb..M1-kb-h+1.
// Unused columns of the last group are transformed but never read.
// The row twiddle table Wl is built while the rows are in flight.
template <int M1, int M2>
__device__ __forceinline__ void p2_group(float2 *sm, float2 *Wl, uint32_t N,
                                         const float2 *__restrict__ in, uint32_t g,
                                         const float2 *__restrict__ Q, int lq,
                                         float *__restrict__ out, double *__restrict__ psum_out) {
  constexpr int C = cols_for(M2), NT = threads_for(M2, C), H = C / 2;
  constexpr uint32_t M = (uint32_t)M1 * M2;
  int h;
  uint32_t kb = 0;
  if (g == 0) {
    h = 1;
  } else {
    kb = 1 + (g - 1) * (uint32_t)H;
    h = (int)min((uint32_t)H, (uint32_t)(M1 / 2 - kb));
  }
  const int ncols = 2 * h;
  const int total = M2 * ncols;
  auto row_of = [&](int ci) -> uint32_t {
    if (g == 0) return ci == 0 ? 0u : (uint32_t)(M1 / 2);
    return ci < h ? kb + (uint32_t)ci : (uint32_t)M1 - (kb + (uint32_t)(ci - h));
  };
  if constexpr (C == 16 && NT == M2) {
    // thread t copies position t of every row to slot lay<16>(t, ci) = 17 t + ci
    const float2 *src = in + threadIdx.x;
    float2 *dst = sm + 17 * threadIdx.x;
#pragma unroll
    for (int ci = 0; ci < C; ++ci)
      if (ci < ncols) cp_async8(dst + ci, src + (uint64_t)row_of(ci) * M2);
    build_wl<M2>(Wl, N, Q, lq);
    cp_async_wait_all();
  } else {
    build_wl<M2>(Wl, N, Q, lq);
#pragma unroll 1
    for (int base = 0; base < total; base += LB * NT) {
      float2 v[LB];
#pragma unroll
      for (int u = 0; u < LB; ++u) {
        const int idx = base + u * NT + (int)threadIdx.x;
        v[u] = idx < total ? in[(uint64_t)row_of(idx / M2) * M2 + idx % M2]
                           : make_float2(0.0f, 0.0f);
      }
#pragma unroll
      for (int u = 0; u < LB; ++u) {
        const int idx = base + u * NT + (int)threadIdx.x;
        if (idx < total) sm[lay<C>(idx % M2, idx / M2)] = v[u];
      }
    }
  }
  __syncthreads();
  const W16 c16 = load_w16<M2>(Wl);
  subfft<M2, C, NT>(sm, Wl, c16);
  Acc2 acc;
  if (g == 0) {
    for (uint32_t idx = threadIdx.x; idx < 2 * M2; idx += NT) {
      const uint32_t k2 = idx % M2, which = idx / M2;
      uint32_t k, mk2;
      if (which == 0) {
        k = M1 * k2;
        mk2 = (M2 - k2) % M2;
      } else {
        k = M1 / 2 + M1 * k2;
        mk2 = M2 - 1 - k2;
      }
      const float p = post_power(sm[lay<C>(k2, which)], sm[lay<C>(mk2, which)], twN(Q, k, lq));
      out[k] = p;
      acc.add(p);
    }
    if (threadIdx.x == 0) {  // k = M (Nyquist): a = Z[0], b = conj(Z[0])
      const float p = post_power(sm[lay<C>(0, 0)], sm[lay<C>(0, 0)], twN(Q, M, lq));
      out[M] = p;
      acc.add(p);
    }
  } else {
    // Bins k = kb + p + M1 k2 and M - k.  W_N^(M-k) = (-W_N^k.re, W_N^k.im)
    // holds bit for bit for the quarter-table lookup (its mirrored half is
    // the swapped first half), up to the sign of zero components, which
    // cannot change |X|^2.  Full groups (h == H) divide by a constant.
    auto rows = [&](auto hc) {
      constexpr int HC = decltype(hc)::value;
      const int hh = HC > 0 ? HC : h;
      constexpr int PB = LB;
      const int tot2 = M2 * hh;
#pragma unroll 1
      for (int base = 0; base < tot2; base += PB * NT) {
        float2 wk[PB];
        uint32_t kk[PB];
        int pp[PB], k2s[PB];
        // Full groups: k2 = t / HC + u NT / HC with t / HC < NT / HC and
        // 4 NT / HC = M2 / 2, so bin k = kb + p + M1 k2 (kb + p < M1 / 2) lies in
        // the first quarter of the quarter-table's cycle for u < 4 and in the
        // second for u >= 4: the quadrant rule of twN, fixed per u.
        constexpr bool QFIX = HC > 0 && PB == 8 && 4 * (NT / (HC > 0 ? HC : 1)) == M2 / 2 &&
                              (HC > 0 ? NT % HC == 0 : false) && M2 * HC == PB * NT;
#pragma unroll
        for (int u = 0; u < PB; ++u) {
          const int idx = base + u * NT + (int)threadIdx.x;
          pp[u] = HC > 0 ? idx % HC : idx % hh;
          k2s[u] = HC > 0 ? idx / HC : idx / hh;
          kk[u] = kb + (uint32_t)pp[u] + M1 * (uint32_t)k2s[u];
          if constexpr (QFIX) {
            if (u < 4) {
              const float2 v = __ldg(&Q[kk[u]]);
              wk[u] = make_float2(v.x, -v.y);
            } else {
              const float2 v = __ldg(&Q[kk[u] - (1u << lq)]);
              wk[u] = make_float2(-v.y, -v.x);
            }
          } else {
            wk[u] = idx < tot2 ? twN(Q, kk[u], lq) : make_float2(1.0f, 0.0f);
          }
        }
#pragma unroll
        for (int u = 0; u < PB; ++u) {
          const int idx = base + u * NT + (int)threadIdx.x;
          if (idx < tot2) {
            const uint32_t k = kk[u];
            const float2 zk = sm[lay<C>(k2s[u], pp[u])];
            const float2 zm = sm[lay<C>(M2 - 1 - k2s[u], hh + pp[u])];
            float pk, pm;
            post_power_pair(zk, zm, wk[u], pk, pm);
            out[k] = pk;
            out[M - k] = pm;
            acc.add(pk);
            acc.add(pm);
          }
        }
      }
    };
    if (h == H) rows(std::integral_constant<int, H>{});
    else rows(std::integral_constant<int, 0>{});
  }
  block_sum_store<NT>(acc, psum_out);
}

// Pass 2: one CTA per row group of every trial.
template <int M1, int M2>
__global__ void __launch_bounds__(threads_for(M2, cols_for(M2)), 2)
    k_fft_pass2(const float2 *__restrict__ work, const float2 *__restrict__ Q, int lq,
                uint32_t N, float *__restrict__ power, uint64_t ldp, double *__restrict__ psum,
                uint32_t ngroups, uint32_t ahead) {
  constexpr int C = cols_for(M2), NT = threads_for(M2, C), H = C / 2;
  constexpr uint32_t M = (uint32_t)M1 * M2;
  extern __shared__ float2 dyn[];
  float2 *Wl = dyn;       // M2 entries
  float2 *sm = dyn + M2;  // lay_slots<M2, C>() entries
  const uint64_t trial = blockIdx.y;
  const uint32_t g = blockIdx.x;
  {
    // Prefetch into L2 the rows of the CTA one resident wave ahead (linear
    // index + ahead): CTAs start roughly in index order, so it runs soon.
    const uint64_t lin = (uint64_t)blockIdx.y * gridDim.x + blockIdx.x + ahead;
    if (ahead && lin < (uint64_t)gridDim.x * gridDim.y) {
      const uint32_t gn = (uint32_t)(lin % gridDim.x);
      const uint64_t tn = lin / gridDim.x;
      const uint32_t kbn = gn == 0 ? 0u : 1 + (gn - 1) * (uint32_t)H;
      const int hn = gn == 0 ? 1 : (int)min((uint32_t)H, (uint32_t)(M1 / 2 - kbn));
      constexpr int LPR = M2 * 8 / 128;  // 128-byte lines per row
      for (int t = threadIdx.x; t < 2 * hn * LPR; t += NT) {
        const int ci = t / LPR;
        const uint32_t k1 = gn == 0 ? (ci == 0 ? 0u : (uint32_t)(M1 / 2))
                                    : (ci < hn ? kbn + (uint32_t)ci
                                               : (uint32_t)M1 - (kbn + (uint32_t)(ci - hn)));
        const float2 *pr = work + tn * M + (uint64_t)k1 * M2 + (t % LPR) * 16;
        asm volatile("prefetch.global.L2 [%0];" ::"l"(pr));
      }
    }
  }
  p2_group<M1, M2>(sm, Wl, N, work + trial * (uint64_t)M, g, Q, lq, power + trial * ldp,
                   psum + trial * ngroups + g);
}

struct FftArgs {
  const float *series;
  uint64_t lds, len;
  const float *means;
  const float2 *Q;
  int lq;
  uint32_t N;
  const float2 *tw1;
  uint64_t ntrials;
  float2 *work;
  float *power;
  uint64_t ldp;
  double *psum;
  cudaStream_t st;
};

// Largest pass-1 dynamic shared memory that keeps two CTAs per SM with the
// staged rows (GB300: 228 KB per SM, 1 KB reserved per CTA, static arrays).
size_t g_pass1_stage_max = 110 * 1024;

// SM count of the current device (cached per device).
int sm_count(int &n) {
  static thread_local int dev_cached = -1, n_cached = 0;
  int dev = 0;
  PSR_CUDA(cudaGetDevice(&dev));
  if (dev != dev_cached) {
    PSR_CUDA(cudaDeviceGetAttribute(&n_cached, cudaDevAttrMultiProcessorCount, dev));
    dev_cached = dev;
  }
  n = n_cached;
  return PSR_OK;
}

template <int M>
int run_small(const FftArgs &a) {
  const size_t smem = (size_t)(M + lay_slots<M, 1>()) * sizeof(float2);
  PSR_CUDA(cudaFuncSetAttribute(k_fft_small<M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem));
  k_fft_small<M><<<(unsigned)a.ntrials, threads_for(M, 1), smem, a.st>>>(
      a.series, a.lds, a.len, a.means, a.Q, a.lq, a.N, a.power, a.ldp, a.psum);
  PSR_CUDA(cudaGetLastError());
  return PSR_OK;
}

template <int M1, int M2>
int run_four_step(const FftArgs &a) {
  {
    constexpr int C = cols_for(M1);
    const size_t smem = (size_t)(M1 + lay_slots<M1, C>()) * sizeof(float2);
    // staged rows: ceil(nz / M2) <= M1 / 2 rows of C complex values (plus the
    // slot that aligns them to 16 bytes)
    const uint64_t rows = ((a.len + 1) / 2 + M2 - 1) / M2;
    const size_t smem_st = smem + (rows * C + 1) * sizeof(float2);
    int nsm = 0;
    PSR_TRY(sm_count(nsm));
    const uint32_t ngroups = (uint32_t)(M2 / C) * (uint32_t)a.ntrials;
    const uint32_t grid = std::min<uint32_t>(ngroups, 2u * (uint32_t)nsm);
    if (C % 2 == 0 && smem_st <= g_pass1_stage_max) {
      PSR_CUDA(cudaFuncSetAttribute(k_fft_pass1<M1, M2, true>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_st));
      k_fft_pass1<M1, M2, true><<<grid, threads_for(M1, C), smem_st, a.st>>>(
          a.series, a.lds, a.len, a.means, a.Q, a.lq, a.N, a.tw1, a.work, ngroups);
    } else {
      PSR_CUDA(cudaFuncSetAttribute(k_fft_pass1<M1, M2, false>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      k_fft_pass1<M1, M2, false><<<grid, threads_for(M1, C), smem, a.st>>>(
          a.series, a.lds, a.len, a.means, a.Q, a.lq, a.N, a.tw1, a.work, ngroups);
    }
    PSR_CUDA(cudaGetLastError());
  }
  {
    constexpr int C = cols_for(M2);
    const size_t smem = (size_t)(M2 + lay_slots<M2, C>()) * sizeof(float2);
    PSR_CUDA(cudaFuncSetAttribute(k_fft_pass2<M1, M2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    const uint32_t ng = 1 + ((uint32_t)M1 / 2 - 1 + C / 2 - 1) / (C / 2);
    dim3 grid(ng, (unsigned)a.ntrials);
    int nsm2 = 0;
    PSR_TRY(sm_count(nsm2));
    k_fft_pass2<M1, M2><<<grid, threads_for(M2, C), smem, a.st>>>(
        a.work, a.Q, a.lq, a.N, a.power, a.ldp, a.psum, ng, 2u * (uint32_t)nsm2);
    PSR_CUDA(cudaGetLastError());
  }
  return PSR_OK;
}

}  // namespace

uint64_t FftPlan::pass2_ctas() const {
  if (m <= 12) return 1;
  const uint32_t C = (uint32_t)(M2 >= 8192 ? 1 : std::min<uint64_t>(16, 8192 / M2));
  const uint32_t H = C / 2;
  return 1 + ((uint32_t)M1 / 2 - 1 + H - 1) / H;
}

int FftPlan::init(uint64_t series_len, cudaStream_t st) {
  if (series_len < 2) {
    set_error("periodicity: series of at least two samples required");
    return PSR_EINVAL;
  }
  uint64_t p = 1;
  while (p < series_len) p <<= 1;
  N = 2 * p;
  M = p;
  if (M > (1ull << 24)) {
    set_error("periodicity: FFT size above 2^25 is not supported");
    return PSR_EINVAL;
  }
  len = series_len;
  m = 0;
  while ((1ull << m) < M) ++m;
  M1 = 1ull << ((m + 1) / 2);
  M2 = 1ull << (m / 2);
  const uint64_t n4 = N / 4, n8 = N / 8;
  std::vector<float2> q(n4 + 1);
  for (uint64_t r = 0; r <= n8; ++r) {
    double a = 6.283185307179586 * (double)r / (double)N;
    q[r] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  for (uint64_t r = n8 + 1; r <= n4; ++r) q[r] = make_float2(q[n4 - r].y, q[n4 - r].x);
  PSR_TRY(Q.ensure(q.size() * sizeof(float2)));
  PSR_CUDA(cudaMemcpyAsync(Q.p, q.data(), q.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
  if (m > 12) {
    // Tw1[k1*M2 + n2] = W_N^(2*n2*k1) = W_M^(n2*k1), from the same quarter table
    // and quadrant rule as the device lookup.
    std::vector<float2> t((size_t)M);
    for (uint64_t k1 = 0; k1 < M1; ++k1)
      for (uint64_t n2 = 0; n2 < M2; ++n2) {
        const uint64_t x = 2 * n2 * k1, qd = x / n4, r = x % n4;
        const float2 v = q[r];
        float2 w;
        switch (qd & 3) {
          case 0: w = make_float2(v.x, -v.y); break;
          case 1: w = make_float2(-v.y, -v.x); break;
          case 2: w = make_float2(-v.x, v.y); break;
          default: w = make_float2(v.y, v.x); break;
        }
        t[k1 * M2 + n2] = w;
      }
    PSR_TRY(tw1.ensure(t.size() * sizeof(float2)));
    PSR_CUDA(cudaMemcpyAsync(tw1.p, t.data(), t.size() * sizeof(float2), cudaMemcpyHostToDevice,
                             st));
  }
  PSR_CUDA(cudaStreamSynchronize(st));
  return PSR_OK;
}

int launch_raw_power_ex(const FftPlan &p, const float *d_series, uint64_t lds,
                        const float *d_means, uint64_t ntrials, float2 *d_work, float *d_power,
                        uint64_t ldp, double *d_psum, cudaStream_t st) {
  int lq = 0;
  while ((1ull << lq) < p.N / 4) ++lq;
  FftArgs a{d_series, lds,          p.len,   d_means, p.Q.as<float2>(), lq, (uint32_t)p.N,
            p.tw1.as<float2>(), ntrials, d_work, d_power, ldp, d_psum, st};
  switch (p.m) {
    case 1: return run_small<2>(a);
    case 2: return run_small<4>(a);
    case 3: return run_small<8>(a);
    case 4: return run_small<16>(a);
    case 5: return run_small<32>(a);
    case 6: return run_small<64>(a);
    case 7: return run_small<128>(a);
    case 8: return run_small<256>(a);
    case 9: return run_small<512>(a);
    case 10: return run_small<1024>(a);
    case 11: return run_small<2048>(a);
    case 12: return run_small<4096>(a);
    case 13: return run_four_step<128, 64>(a);
    case 14: return run_four_step<128, 128>(a);
    case 15: return run_four_step<256, 128>(a);
    case 16: return run_four_step<256, 256>(a);
    case 17: return run_four_step<512, 256>(a);
    case 18: return run_four_step<512, 512>(a);
    case 19: return run_four_step<1024, 512>(a);
    case 20: return run_four_step<1024, 1024>(a);
    case 21: return run_four_step<2048, 1024>(a);
    case 22: return run_four_step<2048, 2048>(a);
    case 23: return run_four_step<4096, 2048>(a);
    case 24: return run_four_step<4096, 4096>(a);
    default:
      set_error("periodicity: unsupported FFT size");
      return PSR_EINVAL;
  }
}

int launch_raw_power_tables(uint64_t len, uint64_t N, const float2 *d_Q, const float2 *d_tw1,
                            const float *d_series, uint64_t lds, const float *d_means,
                            uint64_t ntrials, float2 *d_work, float *d_power, uint64_t ldp,
                            double *d_psum, cudaStream_t st) {
  int lq = 0;
  while ((1ull << lq) < N / 4) ++lq;
  int m = 0;
  while ((1ull << m) < N / 2) ++m;
  FftArgs a{d_series, lds, len, d_means, d_Q, lq, (uint32_t)N, d_tw1, ntrials, d_work, d_power,
            ldp, d_psum, st};
  switch (m) {
    case 1: return run_small<2>(a);
    case 2: return run_small<4>(a);
    case 3: return run_small<8>(a);
    case 4: return run_small<16>(a);
    case 5: return run_small<32>(a);
    case 6: return run_small<64>(a);
    case 7: return run_small<128>(a);
    case 8: return run_small<256>(a);
    case 9: return run_small<512>(a);
    case 10: return run_small<1024>(a);
    case 11: return run_small<2048>(a);
    case 12: return run_small<4096>(a);
    case 13: return run_four_step<128, 64>(a);
    case 14: return run_four_step<128, 128>(a);
    case 15: return run_four_step<256, 128>(a);
    case 16: return run_four_step<256, 256>(a);
    case 17: return run_four_step<512, 256>(a);
    case 18: return run_four_step<512, 512>(a);
    case 19: return run_four_step<1024, 512>(a);
    case 20: return run_four_step<1024, 1024>(a);
    default:
      set_error("periodicity: unsupported FFT size");
      return PSR_EINVAL;
  }
}

}  // namespace psr
