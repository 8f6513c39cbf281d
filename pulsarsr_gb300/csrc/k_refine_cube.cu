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
#include <vector>

#include "psr_internal.h"
#include "refine.h"

namespace psr {
namespace {

constexpr double K_DM_C = 4148.808;  // dedisperse/src/lib.rs:3
constexpr int CB_NT = 256;
constexpr int CB_MAXB = 1024;

// Fold subint s of channel c (one CTA) into C[c][s][*] (the row's mean
// removed, which leaves every shifted profile's deviations unchanged and keeps
// f32 sums accurate) and the channel's sum / sum of squares.  Tiles of
// CB_NT x CB_RUN samples are loaded coalesced into shared memory (one pad word
// per CB_RUN so that per-thread runs are free of bank conflicts); thread j
// then folds the run [j*CB_RUN, (j+1)*CB_RUN) of the tile, its phase anchored
// in f64 at the run's first sample and advanced in f32, summing consecutive
// samples of the same bin in registers and issuing shared-memory atomics only
// when the bin changes (slow pulsars stay in one bin for many samples).
constexpr int CB_RUN = 32;
constexpr int CB_TILE = CB_NT * CB_RUN;

template <class T>
__global__ void __launch_bounds__(CB_NT)
    k_cube_fold(const T *__restrict__ x, uint64_t ld, uint64_t n, int S, int B, double tsamp,
                double nu, double nudot, const double *__restrict__ tau,
                float *__restrict__ cube, double *__restrict__ chsum) {
  __shared__ float bins[CB_MAXB];
  __shared__ float tile[CB_TILE + CB_TILE / CB_RUN];
  __shared__ double red[2][CB_NT / 32];
  __shared__ float mean_s;
  const int s = blockIdx.x;
  const uint64_t c = blockIdx.y;
  for (int b = threadIdx.x; b < B; b += blockDim.x) bins[b] = 0.0f;
  const uint64_t t0 = (n * (uint64_t)s) / (uint64_t)S, t1 = (n * (uint64_t)(s + 1)) / (uint64_t)S;
  const T *row = x + c * ld;
  const double tc = tau[c];
  const float fB = (float)B;
  double sum = 0.0, sq = 0.0;
  for (uint64_t base = t0; base < t1; base += CB_TILE) {
    const int len = (int)min((uint64_t)CB_TILE, t1 - base);
    __syncthreads();  // previous tile consumed (and bins zeroed on entry)
    // At most CB_RUN samples per thread per tile: f32 partial sums (exact for
    // 8-bit samples), one f64 add per tile (the FP64 pipe is narrow).
    float ps = 0.0f, pq = 0.0f;
    for (int i = threadIdx.x; i < len; i += CB_NT) {
      const float v = (float)row[base + i];
      tile[i + i / CB_RUN] = v;
      ps += v;
      pq += v * v;
    }
    sum += (double)ps;
    sq += (double)pq;
    __syncthreads();
    const int r0 = threadIdx.x * CB_RUN;
    if (r0 < len) {
      const int r1 = min(r0 + CB_RUN, len);
      // Phase at the tile start (f64, once per tile and thread, shared
      // expression) plus the run offset: a quadratic in the offset, with the
      // tile's cycles per sample (the f64 pipe is narrow on this GPU).
      const double tdt = (double)base * tsamp - tc;
      const double pht = nu * tdt + 0.5 * nudot * tdt * tdt;
      const double dps_t = (nu + nudot * tdt) * tsamp;  // cycles per sample at the tile start
      const double off = (double)r0;
      const double ph = pht + off * (dps_t + 0.5 * nudot * tsamp * tsamp * off);
      float u = (float)((ph - floor(ph)) * (double)B);
      const double dps = dps_t + nudot * tsamp * tsamp * off;
      const float du = (float)((dps - floor(dps)) * (double)B);
      int cur = -1;
      float a0 = 0.0f, a1 = 0.0f;
      const float *run = tile + threadIdx.x * (CB_RUN + 1);
      for (int i = r0; i < r1; ++i) {
        const float v = run[i - r0];
        float fl = floorf(u);
        int b0 = (int)fl;
        float w = u - fl;
        if (b0 >= B) {
          b0 = 0;
          w = 0.0f;
        }
        if (b0 != cur) {
          if (cur >= 0) {
            atomicAdd(&bins[cur], a0);
            atomicAdd(&bins[cur + 1 == B ? 0 : cur + 1], a1);
          }
          cur = b0;
          a0 = a1 = 0.0f;
        }
        a0 += (1.0f - w) * v;
        a1 += w * v;
        u += du;
        if (u >= fB) u -= fB;
      }
      if (cur >= 0) {
        atomicAdd(&bins[cur], a0);
        atomicAdd(&bins[cur + 1 == B ? 0 : cur + 1], a1);
      }
    }
  }
  for (int o = 16; o; o >>= 1) {
    sum += __shfl_down_sync(0xffffffffu, sum, o);
    sq += __shfl_down_sync(0xffffffffu, sq, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = sum;
    red[1][threadIdx.x >> 5] = sq;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double a = 0.0;
    for (int w2 = 0; w2 < CB_NT / 32; ++w2) a += red[threadIdx.x][w2];
    chsum[(c * (uint64_t)S + (uint64_t)s) * 2 + threadIdx.x] = a;
    if (threadIdx.x == 0) mean_s = (float)(a / (double)B);
  }
  __syncthreads();
  float *dst = cube + (c * (uint64_t)S + (uint64_t)s) * (uint64_t)B;
  for (int b = threadIdx.x; b < B; b += blockDim.x) dst[b] = bins[b] - mean_s;
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

struct CubeWork {
  DevBuf cube, R, chsum, tau, kc, cands, prof, g, grad;
  uint64_t rows = 0;
  double var = 1.0;
};

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
  switch (o.kind) {
    case SAMPLE_U8:
      k_cube_fold<uint8_t><<<grid, CB_NT, 0, st>>>(o.samples.as<uint8_t>(), o.ld, n, S, B,
                                                    o.h.tsamp, nu, nudot, w.tau.as<double>(),
                                                    w.cube.as<float>(), w.chsum.as<double>());
      break;
    case SAMPLE_U16:
      k_cube_fold<uint16_t><<<grid, CB_NT, 0, st>>>(o.samples.as<uint16_t>(), o.ld, n, S, B,
                                                     o.h.tsamp, nu, nudot, w.tau.as<double>(),
                                                     w.cube.as<float>(), w.chsum.as<double>());
      break;
    default:
      k_cube_fold<float><<<grid, CB_NT, 0, st>>>(o.samples.as<float>(), o.ld, n, S, B,
                                                  o.h.tsamp, nu, nudot, w.tau.as<double>(),
                                                  w.cube.as<float>(), w.chsum.as<double>());
  }
  PSR_CUDA(cudaGetLastError());
  PSR_TRY(w.R.ensure(w.rows * (uint64_t)(B / 2) * sizeof(float2)));
  k_cube_dft<<<(unsigned)((w.rows + CB_ROWS - 1) / CB_ROWS), CB_NT, 0, st>>>(
      w.cube.as<float>(), w.rows, B, w.R.as<float2>());
  PSR_CUDA(cudaGetLastError());
  std::vector<double> cs(w.rows * 2);
  PSR_CUDA(cudaMemcpyAsync(cs.data(), w.chsum.p, cs.size() * 8, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  // v = sum over channels of each channel's sample variance (the variance of
  // a sum of independent channels).
  double v = 0.0;
  for (uint64_t c = 0; c < nch; ++c) {
    double s1 = 0.0, s2 = 0.0;
    for (int s = 0; s < S; ++s) {
      s1 += cs[(c * S + s) * 2];
      s2 += cs[(c * S + s) * 2 + 1];
    }
    const double m = s1 / (double)n;
    v += std::fmax(s2 / (double)n - m * m, 0.0);
  }
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

int refine_cube_group(const DeviceObs &o, uint64_t n, const psr_timing *start, uint64_t K,
                      const RefineOptions &opt, psr_timing *out, double *Jout, uint64_t *evals,
                      cudaStream_t st) {
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
  CubeWork w;
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
