// Gradient refinement of (P, Pdot, DM): a differentiable fold objective and
// its hand-written adjoint.  No counterpart in the reference, which refines
// on a grid (fold::refine, fold/src/lib.rs:81-97, and the half-step DM grid of
// search/src/confirmation.rs:295-310); this is the chosen alternative beside
// that grid, not a replacement of it.
//
// Model (all of it computed on the device; FP64 only for phases and the
// parameter-gradient sums):
//   tau_c(DM) = K * DM * (f_c^-2 - f_max^-2) / tsamp = m_c + alpha_c  (samples,
//               m_c = floor, alpha_c in [0,1))
//   y(t)      = sum_c (1 - alpha_c) x[c][t + m_c] + alpha_c x[c][t + m_c + 1]
//               (linear-interpolated fractional-delay dedispersion, f32)
//   phi(t)    = nu T + nu_dot T^2 / 2,  T = t * tsamp, nu = 1/P,
//               nu_dot = -Pdot / P^2
//   u(t)      = B * frac(phi(t)),  b0 = floor(u), w = u - b0, b1 = (b0+1) mod B
//   F[s][b]   : cloud-in-cell fold, F[s][b0] += (1-w) y, F[s][b1] += w y,
//               s = floor(t * S / n)  (subints)
//   p[b]      = sum_s F[s][b],  J = sum_b (p[b] - mean(p))^2 / (n * v)
//               with v the variance of y at the starting point (held fixed).
// Adjoint: g[b] = 2 (p[b] - mean p) / (n v);  per sample
//   dJ/dy(t) = (1-w) g[b0] + w g[b1],  dJ/du(t) = y(t) (g[b1] - g[b0]),
//   dJ/dP    = sum_t dJ/du * B * dphi/dP,  dJ/dPdot likewise,
//   dJ/dDM   = sum_t dJ/dy(t) * z(t),  z(t) = sum_c k_c (x[c][t+m_c+1] - x[c][t+m_c]),
//   k_c      = d tau_c / d DM.
// z is produced by the same pass over the filterbank as y, so one objective
// and gradient evaluation reads the data once.  Subints are folded again at
// every evaluation rather than stored.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "psr_internal.h"
#include "refine.h"

namespace psr {
namespace {

constexpr double K_DM_R = 4148.808;  // dedisperse/src/lib.rs:3
constexpr int RF_NT = 256;
constexpr int RF_TPT = 4;  // samples per thread in the data pass

// y and z for one trial: channel-order f32 sums of interpolated samples.
template <class T>
__global__ void __launch_bounds__(RF_NT)
    k_frac_dedisperse(const T *__restrict__ x, uint64_t ld, uint64_t nch,
                      const int *__restrict__ m, const float *__restrict__ alpha,
                      const float *__restrict__ kc, uint64_t n, float *__restrict__ y,
                      float *__restrict__ z) {
  const uint64_t t0 = ((uint64_t)blockIdx.x * RF_TPT) * RF_NT + threadIdx.x;
  float ay[RF_TPT], az[RF_TPT];
#pragma unroll
  for (int i = 0; i < RF_TPT; ++i) ay[i] = az[i] = 0.0f;
  for (uint64_t c = 0; c < nch; ++c) {
    const T *row = x + c * ld + m[c];
    const float a = alpha[c], b = 1.0f - a, k = kc[c];
#pragma unroll
    for (int i = 0; i < RF_TPT; ++i) {
      const uint64_t t = t0 + (uint64_t)i * RF_NT;
      if (t < n) {
        const float v0 = (float)row[t], v1 = (float)row[t + 1];
        ay[i] = __fadd_rn(ay[i], __fadd_rn(__fmul_rn(b, v0), __fmul_rn(a, v1)));
        az[i] = __fadd_rn(az[i], __fmul_rn(k, __fsub_rn(v1, v0)));
      }
    }
  }
#pragma unroll
  for (int i = 0; i < RF_TPT; ++i) {
    const uint64_t t = t0 + (uint64_t)i * RF_NT;
    if (t < n) {
      y[t] = ay[i];
      z[t] = az[i];
    }
  }
}

struct PhaseArgs {
  double tsamp, nu, nudot;
  int bins, subints;
  uint64_t n;
};

__device__ __forceinline__ void phase_of(const PhaseArgs &a, uint64_t t, int &b0, int &b1,
                                         double &w, int &s) {
  const double T = (double)t * a.tsamp;
  const double ph = a.nu * T + 0.5 * a.nudot * T * T;
  const double u = (ph - floor(ph)) * (double)a.bins;
  double fb = floor(u);
  b0 = (int)fb;
  w = u - fb;
  if (b0 >= a.bins) {  // u rounded up to B
    b0 = 0;
    w = 0.0;
  }
  b1 = b0 + 1 == a.bins ? 0 : b0 + 1;
  s = (int)((t * (uint64_t)a.subints) / a.n);
}

// Cloud-in-cell fold into per-CTA shared (subint, bin) accumulators; each CTA
// covers a contiguous range of samples, so it touches at most two subints in
// practice but the shared array holds all S*B cells.
__global__ void __launch_bounds__(RF_NT)
    k_cic_fold(const float *__restrict__ y, PhaseArgs a, uint64_t per_cta,
               double *__restrict__ parts) {
  extern __shared__ double cell[];
  const int cells = a.bins * a.subints;
  for (int i = threadIdx.x; i < cells; i += blockDim.x) cell[i] = 0.0;
  __syncthreads();
  const uint64_t t0 = (uint64_t)blockIdx.x * per_cta;
  const uint64_t t1 = min(t0 + per_cta, a.n);
  for (uint64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
    int b0, b1, s;
    double w;
    phase_of(a, t, b0, b1, w, s);
    const double v = (double)y[t];
    atomicAdd(&cell[s * a.bins + b0], (1.0 - w) * v);
    atomicAdd(&cell[s * a.bins + b1], w * v);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < cells; i += blockDim.x)
    parts[(uint64_t)blockIdx.x * cells + i] = cell[i];
}

__global__ void k_sum_parts(const double *__restrict__ parts, uint64_t nparts, int cells,
                            double *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cells) return;
  double s = 0.0;
  for (uint64_t p = 0; p < nparts; ++p) s += parts[p * cells + i];
  out[i] = s;
}

// Per-CTA partial sums of dJ/dnu, dJ/dnudot, dJ/dDM and of y, y^2.
__global__ void __launch_bounds__(RF_NT)
    k_adjoint(const float *__restrict__ y, const float *__restrict__ z,
              const double *__restrict__ g, PhaseArgs a, double *__restrict__ parts) {
  __shared__ double red[5][RF_NT / 32];
  double acc[5] = {0, 0, 0, 0, 0};
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < a.n;
       t += (uint64_t)gridDim.x * blockDim.x) {
    int b0, b1, s;
    double w;
    phase_of(a, t, b0, b1, w, s);
    const double v = (double)y[t];
    const double gb0 = g[b0], gb1 = g[b1];
    const double dy = (1.0 - w) * gb0 + w * gb1;  // dJ/dy(t)
    const double du = v * (gb1 - gb0);            // dJ/du(t)
    const double T = (double)t * a.tsamp;
    acc[0] += du * T;            // dJ/dnu / B
    acc[1] += du * 0.5 * T * T;  // dJ/dnudot / B
    acc[2] += dy * (double)z[t];
    acc[3] += v;
    acc[4] += v * v;
  }
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    double x = acc[j];
    for (int o = 16; o; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) red[j][threadIdx.x >> 5] = x;
  }
  __syncthreads();
  if (threadIdx.x < 5) {
    double x = 0.0;
    for (int w2 = 0; w2 < RF_NT / 32; ++w2) x += red[threadIdx.x][w2];
    parts[blockIdx.x * 5 + threadIdx.x] = x;
  }
}

}  // namespace

int RefineWork::evaluate(const DeviceObs &o, uint64_t n, const psr_timing &th,
                         const RefineOptions &opt, double v_fixed, RefineEval &ev,
                         cudaStream_t st) {
  const uint64_t nch = o.nch;
  const double tsamp = o.h.tsamp;
  if (!(th.period_s > 0.0) || !std::isfinite(th.period_s) || !std::isfinite(th.pdot) ||
      !(th.dm >= 0.0) || !std::isfinite(th.dm)) {
    set_error("refine: finite positive period, finite pdot and nonnegative DM required");
    return PSR_EINVAL;
  }
  // Fractional delays (FP64 on the host, as the integer delay tables).
  double fmax = 0.0;
  for (uint64_t c = 0; c < nch; ++c) fmax = std::fmax(fmax, o.h.fch1 + (double)c * o.h.foff);
  std::vector<int> m(nch);
  std::vector<float> alpha(nch), kc(nch);
  int mmax = 0;
  for (uint64_t c = 0; c < nch; ++c) {
    const double f = o.h.fch1 + (double)c * o.h.foff;
    const double k = K_DM_R * (1.0 / (f * f) - 1.0 / (fmax * fmax)) / tsamp;
    const double tau = k * th.dm;
    const double fl = std::floor(tau);
    m[c] = (int)fl;
    alpha[c] = (float)(tau - fl);
    kc[c] = (float)k;
    mmax = std::max(mmax, m[c]);
  }
  if ((uint64_t)mmax + n + 1 > o.ns) {
    set_error("refine: the DM's delays leave fewer than n + 1 samples");
    return PSR_EDEDISPERSE;
  }
  PSR_TRY(dm_.ensure(nch * 4));
  PSR_TRY(dalpha_.ensure(nch * 4));
  PSR_TRY(dk_.ensure(nch * 4));
  PSR_TRY(y_.ensure(n * 4 + 16));
  PSR_TRY(z_.ensure(n * 4 + 16));
  PSR_CUDA(cudaMemcpyAsync(dm_.p, m.data(), nch * 4, cudaMemcpyHostToDevice, st));
  PSR_CUDA(cudaMemcpyAsync(dalpha_.p, alpha.data(), nch * 4, cudaMemcpyHostToDevice, st));
  PSR_CUDA(cudaMemcpyAsync(dk_.p, kc.data(), nch * 4, cudaMemcpyHostToDevice, st));
  const unsigned gx = (unsigned)((n + RF_NT * RF_TPT - 1) / (RF_NT * RF_TPT));
  switch (o.kind) {
    case SAMPLE_U8:
      k_frac_dedisperse<uint8_t><<<gx, RF_NT, 0, st>>>(
          o.samples.as<uint8_t>(), o.ld, nch, dm_.as<int>(), dalpha_.as<float>(),
          dk_.as<float>(), n, y_.as<float>(), z_.as<float>());
      break;
    case SAMPLE_U16:
      k_frac_dedisperse<uint16_t><<<gx, RF_NT, 0, st>>>(
          o.samples.as<uint16_t>(), o.ld, nch, dm_.as<int>(), dalpha_.as<float>(),
          dk_.as<float>(), n, y_.as<float>(), z_.as<float>());
      break;
    default:
      k_frac_dedisperse<float><<<gx, RF_NT, 0, st>>>(
          o.samples.as<float>(), o.ld, nch, dm_.as<int>(), dalpha_.as<float>(),
          dk_.as<float>(), n, y_.as<float>(), z_.as<float>());
  }
  PSR_CUDA(cudaGetLastError());
  const int B = (int)opt.bins, S = (int)opt.subints;
  const int cells = B * S;
  PhaseArgs a{tsamp, 1.0 / th.period_s, -th.pdot / (th.period_s * th.period_s), B, S, n};
  const uint64_t per_cta = 16384;
  const uint64_t nparts = (n + per_cta - 1) / per_cta;
  if (cells * 8 > 160 * 1024) {
    set_error("refine: bins * subints must stay below 20480");
    return PSR_EINVAL;
  }
  PSR_TRY(parts_.ensure(nparts * cells * 8));
  PSR_TRY(cells_.ensure(cells * 8));
  PSR_CUDA(cudaFuncSetAttribute(k_cic_fold, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                cells * 8));
  k_cic_fold<<<(unsigned)nparts, RF_NT, cells * 8, st>>>(y_.as<float>(), a, per_cta,
                                                          parts_.as<double>());
  PSR_CUDA(cudaGetLastError());
  k_sum_parts<<<(cells + 255) / 256, 256, 0, st>>>(parts_.as<double>(), nparts, cells,
                                                    cells_.as<double>());
  PSR_CUDA(cudaGetLastError());
  ev.cells.resize(cells);
  PSR_CUDA(cudaMemcpyAsync(ev.cells.data(), cells_.p, cells * 8, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  // Profile, objective and the adjoint seed g on the host (B values).
  std::vector<double> p(B, 0.0);
  for (int s = 0; s < S; ++s)
    for (int b = 0; b < B; ++b) p[b] += ev.cells[(size_t)s * B + b];
  double mean = 0.0;
  for (double x : p) mean += x;
  mean /= (double)B;
  const double norm = (double)n * v_fixed;
  double J = 0.0;
  std::vector<double> g(B);
  for (int b = 0; b < B; ++b) {
    const double d = p[b] - mean;
    J += d * d;
    g[b] = 2.0 * d / norm;
  }
  ev.J = J / norm;
  ev.profile = p;
  PSR_TRY(g_.ensure(B * 8));
  PSR_CUDA(cudaMemcpyAsync(g_.p, g.data(), B * 8, cudaMemcpyHostToDevice, st));
  const unsigned ga = (unsigned)std::min<uint64_t>((n + RF_NT - 1) / RF_NT, 1216);
  PSR_TRY(adj_.ensure(ga * 5 * 8));
  k_adjoint<<<ga, RF_NT, 0, st>>>(y_.as<float>(), z_.as<float>(), g_.as<double>(), a,
                                  adj_.as<double>());
  PSR_CUDA(cudaGetLastError());
  std::vector<double> h((size_t)ga * 5);
  PSR_CUDA(cudaMemcpyAsync(h.data(), adj_.p, h.size() * 8, cudaMemcpyDeviceToHost, st));
  PSR_CUDA(cudaStreamSynchronize(st));
  double s5[5] = {0, 0, 0, 0, 0};
  for (unsigned i = 0; i < ga; ++i)
    for (int j = 0; j < 5; ++j) s5[j] += h[(size_t)i * 5 + j];
  // Chain rule from (nu, nudot) to (P, Pdot): nu = 1/P, nudot = -Pdot/P^2.
  const double dnu = s5[0] * (double)B, dnudot = s5[1] * (double)B;
  const double P = th.period_s;
  ev.dnu = dnu;
  ev.dnudot = dnudot;
  ev.dP = dnu * (-1.0 / (P * P)) + dnudot * (2.0 * th.pdot / (P * P * P));
  ev.dPdot = dnudot * (-1.0 / (P * P));
  ev.dDM = s5[2];
  ev.mean_y = s5[3] / (double)n;
  ev.var_y = std::fmax(s5[4] / (double)n - ev.mean_y * ev.mean_y, 0.0);
  return PSR_OK;
}

// Largest DM whose delays keep n + 1 samples inside the observation.
double max_dm_for(const DeviceObs &o, uint64_t n) {
  double fmax = 0.0, fmin = 1e300;
  for (uint64_t c = 0; c < o.nch; ++c) {
    const double f = o.h.fch1 + (double)c * o.h.foff;
    fmax = std::fmax(fmax, f);
    fmin = std::fmin(fmin, f);
  }
  const double k = K_DM_R * (1.0 / (fmin * fmin) - 1.0 / (fmax * fmax)) / o.h.tsamp;
  if (!(k > 0.0) || n + 2 > o.ns) return 0.0;
  return ((double)(o.ns - n - 2)) / k;
}

int refine_gradient_one(const DeviceObs &o, uint64_t n, const psr_timing &start,
                        const RefineOptions &opt, RefineWork &w, psr_timing &out, double &J,
                        uint64_t &evals, cudaStream_t st) {
  const double B = (double)opt.bins;
  const double T = (double)n * o.h.tsamp;
  double fmax = 0.0, fmin = 1e300;
  for (uint64_t c = 0; c < o.nch; ++c) {
    const double f = o.h.fch1 + (double)c * o.h.foff;
    fmax = std::fmax(fmax, f);
    fmin = std::fmin(fmin, f);
  }
  const double kspan = K_DM_R * (1.0 / (fmin * fmin) - 1.0 / (fmax * fmax));  // s per DM
  const double nu0 = 1.0 / start.period_s;
  const double nudot0 = -start.pdot / (start.period_s * start.period_s);
  // Scaled coordinates (one unit = one profile bin), orthogonal over the
  // span: with x = 2T/T_end - 1 the phase change is q1 x / B + q2 (x^2 - 1/3) / B,
  // i.e. dnu = (2 q1 - 4 q2) / (B T_end), dnudot = 8 q2 / (B T_end^2); q3 moves
  // the lowest channel's phase by q3 bins through DM.
  const double s3 = kspan > 0.0 ? start.period_s / (B * kspan) : 1.0;
  const double dm_hi = max_dm_for(o, n);
  auto theta = [&](const double q[3]) {
    const double nu = nu0 + (2.0 * q[0] - 4.0 * q[1]) / (B * T);
    const double nudot = nudot0 + 8.0 * q[1] / (B * T * T);
    psr_timing t;
    t.period_s = 1.0 / nu;
    t.pdot = -nudot / (nu * nu);
    double dm = start.dm + q[2] * s3;
    if (opt.dm_window > 0.0)
      dm = std::fmin(std::fmax(dm, start.dm - opt.dm_window), start.dm + opt.dm_window);
    t.dm = std::fmin(std::fmax(dm, 0.0), dm_hi);
    return t;
  };
  RefineEval ev;
  evals = 0;
  double q[3] = {0, 0, 0};
  PSR_TRY(w.evaluate(o, n, theta(q), opt, 1.0, ev, st));
  ++evals;
  const double v = ev.var_y > 0.0 ? ev.var_y : 1.0;
  auto grad_q = [&](const RefineEval &e, double g[3]) {
    g[0] = e.dnu * 2.0 / (B * T);
    g[1] = e.dnu * (-4.0 / (B * T)) + e.dnudot * 8.0 / (B * T * T);
    g[2] = e.dDM * s3;
  };
  double Jc = ev.J / v, g[3];
  grad_q(ev, g);
  for (double &x : g) x /= v;
  double H[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  const double gn = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
  const double h0 = gn > 0.0 ? 1.0 / gn : 1.0;  // first step: one bin
  for (int i = 0; i < 3; ++i) H[i][i] = h0;
  while (evals < opt.max_evals) {
    double d[3];
    for (int i = 0; i < 3; ++i) d[i] = H[i][0] * g[0] + H[i][1] * g[1] + H[i][2] * g[2];
    double slope = d[0] * g[0] + d[1] * g[1] + d[2] * g[2];
    if (!(slope > 0.0)) {  // not an ascent direction: restart from the gradient
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) H[i][j] = i == j ? h0 : 0.0;
      for (int i = 0; i < 3; ++i) d[i] = h0 * g[i];
      slope = h0 * (g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
      if (!(slope > 0.0)) break;
    }
    double alpha = 1.0, qn[3], Jn = -INFINITY, gnew[3] = {0, 0, 0};
    bool accepted = false;
    for (int ls = 0; ls < 12 && evals < opt.max_evals; ++ls) {
      for (int i = 0; i < 3; ++i) qn[i] = q[i] + alpha * d[i];
      RefineEval e2;
      PSR_TRY(w.evaluate(o, n, theta(qn), opt, v, e2, st));
      ++evals;
      if (e2.J >= Jc + 1e-4 * alpha * slope) {
        Jn = e2.J;
        grad_q(e2, gnew);
        accepted = true;
        break;
      }
      alpha *= 0.5;
    }
    if (!accepted) break;
    double sv[3], yv[3];
    double maxstep = 0.0;
    for (int i = 0; i < 3; ++i) {
      sv[i] = qn[i] - q[i];
      yv[i] = -(gnew[i] - g[i]);  // gradient change of -J
      maxstep = std::fmax(maxstep, std::fabs(sv[i]));
    }
    const double sy = sv[0] * yv[0] + sv[1] * yv[1] + sv[2] * yv[2];
    if (sy > 1e-12) {  // BFGS update of the inverse Hessian of -J
      double Hy[3], yHy = 0.0;
      for (int i = 0; i < 3; ++i) Hy[i] = H[i][0] * yv[0] + H[i][1] * yv[1] + H[i][2] * yv[2];
      for (int i = 0; i < 3; ++i) yHy += yv[i] * Hy[i];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          H[i][j] += (sy + yHy) * sv[i] * sv[j] / (sy * sy) - (Hy[i] * sv[j] + sv[i] * Hy[j]) / sy;
    }
    for (int i = 0; i < 3; ++i) {
      q[i] = qn[i];
      g[i] = gnew[i];
    }
    Jc = Jn;
    if (maxstep < opt.tol) break;
  }
  out = theta(q);
  J = Jc;
  return PSR_OK;
}

}  // namespace psr

// ------------------------------------------------------------------ C ABI
extern "C" void psr_refine_options_default(psr_refine_options *out) {
  if (out) *out = psr_refine_options{128, 64, 40, 1e-3, 0, 0.0};
}
