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
// A CTA transforms C columns held in shared memory as [position][C+1]
// (padding keeps both the row-wise global loads and the Stockham accesses
// free of bank conflicts).  All stages are in place: every thread loads its
// butterflies' inputs, the block synchronises, then stores.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "psr_internal.h"

namespace psr {
namespace {

constexpr int LB = 16;  // loads in flight per thread when staging a tile
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

__device__ __forceinline__ void dft2(float2 *v) {
  float2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}
__device__ __forceinline__ void dft4(float2 &v0, float2 &v1, float2 &v2, float2 &v3) {
  float2 a = cadd(v0, v2), b = csub(v0, v2);
  float2 c = cadd(v1, v3), d = mul_mi(csub(v1, v3));
  v0 = cadd(a, c);
  v1 = cadd(b, d);
  v2 = csub(a, c);
  v3 = csub(b, d);
}
// Wl[y] = W_L^y; W_R^y = Wl[y * L / R].
__device__ __forceinline__ void dft8(float2 *v, const float2 *Wl, int L) {
  float2 u[4][2];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    float2 t[2] = {v[n2], v[n2 + 4]};
    dft2(t);
    u[n2][0] = t[0];
    u[n2][1] = t[1];
  }
#pragma unroll
  for (int n2 = 1; n2 < 4; ++n2) u[n2][1] = cmul(u[n2][1], Wl[n2 * (L / 8)]);
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
__device__ __forceinline__ void dft16(float2 *v, const float2 *Wl, int L) {
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
#pragma unroll
  for (int n2 = 1; n2 < 4; ++n2)
#pragma unroll
    for (int k1 = 1; k1 < 4; ++k1) u[n2][k1] = cmul(u[n2][k1], Wl[n2 * k1 * (L / 16)]);
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
__device__ __forceinline__ void dftR(float2 *v, const float2 *Wl, int L) {
  if constexpr (R == 2) dft2(v);
  else if constexpr (R == 4) dft4(v[0], v[1], v[2], v[3]);
  else if constexpr (R == 8) dft8(v, Wl, L);
  else dft16(v, Wl, L);
}

// One in-place Stockham stage on C columns of length L (stride S).
template <int R>
__device__ void stockham_stage(float2 *sm, int S, int C, int L, int Ns, const float2 *Wl) {
  constexpr int BPT = 16 / R;  // butterflies per thread (nthreads >= L/16 * C)
  const int nb = L / R;
  const int total = nb * C;
  float2 v[BPT][R];
  int jj[BPT], cc[BPT];
#pragma unroll
  for (int i = 0; i < BPT; ++i) {
    const int w = threadIdx.x + i * blockDim.x;
    jj[i] = -1;
    if (w < total) {
      const int col = w % C, j = w / C;
      jj[i] = j;
      cc[i] = col;
#pragma unroll
      for (int r = 0; r < R; ++r) v[i][r] = sm[(j + r * nb) * S + col];
      const int k = j & (Ns - 1);
      if (Ns > 1 && k != 0) {
        const int step = L / (Ns * R);
#pragma unroll
        for (int r = 1; r < R; ++r) v[i][r] = cmul(v[i][r], Wl[r * k * step]);
      }
      dftR<R>(v[i], Wl, L);
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < BPT; ++i) {
    if (jj[i] >= 0) {
      const int j = jj[i], k = j & (Ns - 1);
      const int base = (j / Ns) * Ns * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) sm[(base + r * Ns) * S + cc[i]] = v[i][r];
    }
  }
  __syncthreads();
}

__device__ void subfft(float2 *sm, int S, int C, int L, const float2 *Wl) {
  int q = 0;
  while ((1 << q) < L) ++q;
  int Ns = 1;
  for (int s = 0; s < q / 4; ++s) {
    stockham_stage<16>(sm, S, C, L, Ns, Wl);
    Ns *= 16;
  }
  switch (q % 4) {
    case 1: stockham_stage<2>(sm, S, C, L, Ns, Wl); break;
    case 2: stockham_stage<4>(sm, S, C, L, Ns, Wl); break;
    case 3: stockham_stage<8>(sm, S, C, L, Ns, Wl); break;
    default: break;
  }
}

__device__ void build_wl(float2 *Wl, int L, uint32_t N, const float2 *Q, int lq) {
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

__device__ __forceinline__ float trial_mean(const double *sums, uint64_t trial, uint64_t len) {
  return (float)(sums[trial] / (double)len);
}

// Whole transform in one CTA per trial (M <= 4096).
__global__ void __launch_bounds__(512) k_fft_small(const float *__restrict__ series, uint64_t lds, uint64_t len,
                            const double *__restrict__ sums, const float2 *__restrict__ Q,
                            int lq, uint32_t N, uint32_t M, float *__restrict__ power,
                            uint64_t ldp, double *__restrict__ psum) {
  extern __shared__ float2 dyn[];
  float2 *Wl = dyn;          // M entries
  float2 *sm = dyn + M;      // M x 2 (C = 1, S = 2)
  const uint64_t trial = blockIdx.x;
  const float *row = series + trial * lds;
  const float mean = trial_mean(sums, trial, len);
  build_wl(Wl, (int)M, N, Q, lq);
  for (uint32_t n = threadIdx.x; n < M; n += blockDim.x) sm[n * 2] = load_z(row, len, n, mean);
  __syncthreads();
  subfft(sm, 2, 1, (int)M, Wl);
  double acc = 0.0;
  float *out = power + trial * ldp;
  for (uint32_t k = threadIdx.x; k <= M; k += blockDim.x) {
    const float p = post_power(sm[(k % M) * 2], sm[((M - k) % M) * 2], twN(Q, k, lq));
    out[k] = p;
    acc += (double)p;
  }
  __shared__ double red[32];
  for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)((blockDim.x + 31) / 32); ++w) t += red[w];
    psum[trial] = t;
  }
}

// Pass 1: C columns n2 in [n2_0, n2_0 + C) of length M1, then W_M^(n2*k1).
__global__ void __launch_bounds__(512) k_fft_pass1(const float *__restrict__ series, uint64_t lds, uint64_t len,
                            const double *__restrict__ sums, const float2 *__restrict__ Q,
                            int lq, uint32_t N, uint32_t M, uint32_t M1, uint32_t M2, int C,
                            float2 *__restrict__ work) {
  extern __shared__ float2 dyn[];
  float2 *Wl = dyn;        // M1 entries
  float2 *sm = dyn + M1;   // M1 x (C+1)
  const int S = C + 1;
  const uint64_t trial = blockIdx.y;
  const uint32_t n2_0 = blockIdx.x * (uint32_t)C;
  const float *row = series + trial * lds;
  const float mean = trial_mean(sums, trial, len);
  build_wl(Wl, (int)M1, N, Q, lq);
  const uint64_t nz = (len + 1) / 2;  // complex inputs that can be non-zero
  const int total = (int)M1 * C;
  // Batches of LB independent loads per thread keep many requests in flight.
  for (int base = 0; base < total; base += LB * (int)blockDim.x) {
    float2 v[LB];
#pragma unroll
    for (int u = 0; u < LB; ++u) {
      const int idx = base + u * (int)blockDim.x + (int)threadIdx.x;
      const uint64_t n = (uint64_t)(idx / C) * M2 + n2_0 + (idx % C);
      v[u] = (idx < total && n < nz) ? load_z(row, len, n, mean) : make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int u = 0; u < LB; ++u) {
      const int idx = base + u * (int)blockDim.x + (int)threadIdx.x;
      if (idx < total) sm[(idx / C) * S + (idx % C)] = v[u];
    }
  }
  __syncthreads();
  subfft(sm, S, C, (int)M1, Wl);
  float2 *out = work + trial * (uint64_t)M;
  // Twiddle loads for LB outputs are issued before any is consumed.
  for (int base = 0; base < total; base += LB * (int)blockDim.x) {
    float2 w[LB];
#pragma unroll
    for (int u = 0; u < LB; ++u) {
      const int idx = base + u * (int)blockDim.x + (int)threadIdx.x;
      const uint32_t e = (n2_0 + (uint32_t)(idx % C)) * (uint32_t)(idx / C);
      w[u] = (idx < total && e != 0) ? twN(Q, 2u * e, lq) : make_float2(1.0f, 0.0f);
    }
#pragma unroll
    for (int u = 0; u < LB; ++u) {
      const int idx = base + u * (int)blockDim.x + (int)threadIdx.x;
      if (idx < total) {
        const int col = idx % C, k1 = idx / C;
        const uint32_t n2 = n2_0 + (uint32_t)col;
        float2 v = sm[k1 * S + col];
        if (n2 * (uint32_t)k1 != 0) v = cmul(v, w[u]);
        out[(uint64_t)k1 * M2 + n2] = v;
      }
    }
  }
}

// Pass 2: row sub-FFTs of length M2 for a group of rows and their mirrors,
// then the real post-processing and |X|^2.  Group 0 holds rows 0 and M1/2;
// group g >= 1 holds rows kb..kb+h-1 (kb = 1 + (g-1)*H) and M1-kb..M1-kb-h+1.
__global__ void __launch_bounds__(512) k_fft_pass2(const float2 *__restrict__ work, const float2 *__restrict__ Q,
                            int lq, uint32_t N, uint32_t M, uint32_t M1, uint32_t M2, int C,
                            float *__restrict__ power, uint64_t ldp,
                            double *__restrict__ psum, uint32_t ngroups) {
  extern __shared__ float2 dyn[];
  float2 *Wl = dyn;        // M2 entries
  float2 *sm = dyn + M2;   // M2 x (C+1)
  const int S = C + 1;
  const int H = C / 2;
  const uint64_t trial = blockIdx.y;
  const uint32_t g = blockIdx.x;
  const float2 *in = work + trial * (uint64_t)M;
  float *out = power + trial * ldp;
  int h;
  uint32_t kb = 0;
  if (g == 0) {
    h = 1;
  } else {
    kb = 1 + (g - 1) * (uint32_t)H;
    h = (int)min((uint32_t)H, (uint32_t)(M1 / 2 - kb));
  }
  const int ncols = 2 * h;
  build_wl(Wl, (int)M2, N, Q, lq);
  const int total = (int)M2 * ncols;
  for (int base = 0; base < total; base += LB * (int)blockDim.x) {
    float2 v[LB];
#pragma unroll
    for (int u = 0; u < LB; ++u) {
      const int idx = base + u * (int)blockDim.x + (int)threadIdx.x;
      const int pos = idx % (int)M2, ci = idx / (int)M2;
      uint32_t k1;
      if (g == 0) k1 = ci == 0 ? 0 : M1 / 2;
      else k1 = ci < h ? kb + ci : M1 - (kb + (ci - h));
      v[u] = idx < total ? in[(uint64_t)k1 * M2 + pos] : make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int u = 0; u < LB; ++u) {
      const int idx = base + u * (int)blockDim.x + (int)threadIdx.x;
      if (idx < total) sm[(idx % (int)M2) * S + idx / (int)M2] = v[u];
    }
  }
  __syncthreads();
  subfft(sm, S, ncols, (int)M2, Wl);
  double acc = 0.0;
  if (g == 0) {
    for (uint32_t idx = threadIdx.x; idx < 2 * M2; idx += blockDim.x) {
      const uint32_t k2 = idx % M2, which = idx / M2;
      uint32_t k, mk2;
      if (which == 0) {
        k = M1 * k2;
        mk2 = (M2 - k2) % M2;
      } else {
        k = M1 / 2 + M1 * k2;
        mk2 = M2 - 1 - k2;
      }
      const float p = post_power(sm[k2 * S + which], sm[mk2 * S + which], twN(Q, k, lq));
      out[k] = p;
      acc += (double)p;
    }
    if (threadIdx.x == 0) {  // k = M (Nyquist): a = Z[0], b = conj(Z[0])
      const float p = post_power(sm[0], sm[0], twN(Q, M, lq));
      out[M] = p;
      acc += (double)p;
    }
  } else {
    constexpr int PB = LB / 2;  // bins per batch (two twiddles each)
    const int tot2 = (int)M2 * h;
    for (int base = 0; base < tot2; base += PB * (int)blockDim.x) {
      float2 wk[PB], wm[PB];
#pragma unroll
      for (int u = 0; u < PB; ++u) {
        const int idx = base + u * (int)blockDim.x + (int)threadIdx.x;
        const uint32_t k = kb + (uint32_t)(idx % h) + M1 * (uint32_t)(idx / h);
        const bool in = idx < tot2;
        wk[u] = in ? twN(Q, k, lq) : make_float2(1.0f, 0.0f);
        wm[u] = in ? twN(Q, M - k, lq) : make_float2(1.0f, 0.0f);
      }
#pragma unroll
      for (int u = 0; u < PB; ++u) {
        const int idx = base + u * (int)blockDim.x + (int)threadIdx.x;
        if (idx < tot2) {
          const int p = idx % h;
          const uint32_t k2 = (uint32_t)(idx / h);
          const uint32_t k = kb + (uint32_t)p + M1 * k2;
          const uint32_t mk = M - k;
          const float2 zk = sm[k2 * S + p];
          const float2 zm = sm[(M2 - 1 - k2) * S + h + p];
          const float pk = post_power(zk, zm, wk[u]);
          const float pm = post_power(zm, zk, wm[u]);
          out[k] = pk;
          out[mk] = pm;
          acc += (double)pk + (double)pm;
        }
      }
    }
  }
  __shared__ double red[32];
  for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)((blockDim.x + 31) / 32); ++w) t += red[w];
    psum[trial * ngroups + g] = t;
  }
}

int cols_for(uint32_t L) {
  int c = (int)(8192u / L);
  if (c > 16) c = 16;
  if (c < 1) c = 1;
  return c;
}
int threads_for(uint32_t L, int C) {
  int t = (int)(L / 16) * C;
  if (t < 32) t = 32;
  return ((t + 31) / 32) * 32;
}

}  // namespace

uint64_t FftPlan::pass2_ctas() const {
  if (m <= 12) return 1;
  const int C = cols_for((uint32_t)M2);
  const uint32_t H = (uint32_t)C / 2;
  const uint32_t rest = (uint32_t)M1 / 2 - 1;
  return 1 + (rest + H - 1) / H;
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
  PSR_CUDA(cudaStreamSynchronize(st));
  return PSR_OK;
}

int launch_raw_power_ex(const FftPlan &p, const float *d_series, uint64_t lds,
                        const double *d_sums, uint64_t ntrials, float2 *d_work, float *d_power,
                        uint64_t ldp, double *d_psum, cudaStream_t st) {
  int lq = 0;
  while ((1ull << lq) < p.N / 4) ++lq;
  const float2 *Q = p.Q.as<float2>();
  if (p.m <= 12) {
    const int thr = threads_for((uint32_t)p.M, 1);
    const size_t smem = (size_t)p.M * sizeof(float2) * 3;
    PSR_CUDA(cudaFuncSetAttribute(k_fft_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    k_fft_small<<<(unsigned)ntrials, thr, smem, st>>>(d_series, lds, p.len, d_sums, Q, lq,
                                                     (uint32_t)p.N, (uint32_t)p.M, d_power,
                                                     ldp, d_psum);
    PSR_CUDA(cudaGetLastError());
    return PSR_OK;
  }
  {
    const int C = cols_for((uint32_t)p.M1);
    const int thr = threads_for((uint32_t)p.M1, C);
    const size_t smem = (size_t)p.M1 * sizeof(float2) * (1 + C + 1);
    PSR_CUDA(cudaFuncSetAttribute(k_fft_pass1, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    dim3 grid((unsigned)(p.M2 / C), (unsigned)ntrials);
    k_fft_pass1<<<grid, thr, smem, st>>>(d_series, lds, p.len, d_sums, Q, lq, (uint32_t)p.N,
                                         (uint32_t)p.M, (uint32_t)p.M1, (uint32_t)p.M2, C,
                                         d_work);
    PSR_CUDA(cudaGetLastError());
  }
  {
    const int C = cols_for((uint32_t)p.M2);
    const int thr = threads_for((uint32_t)p.M2, C);
    const size_t smem = (size_t)p.M2 * sizeof(float2) * (1 + C + 1);
    PSR_CUDA(cudaFuncSetAttribute(k_fft_pass2, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    const uint32_t ng = (uint32_t)p.pass2_ctas();
    dim3 grid(ng, (unsigned)ntrials);
    k_fft_pass2<<<grid, thr, smem, st>>>(d_work, Q, lq, (uint32_t)p.N, (uint32_t)p.M,
                                         (uint32_t)p.M1, (uint32_t)p.M2, C, d_power, ldp,
                                         d_psum, ng);
    PSR_CUDA(cudaGetLastError());
  }
  return PSR_OK;
}

}  // namespace psr
