// Gradient refinement internals (k_refine.cu).
#pragma once
#include <vector>

#include "psr_internal.h"

namespace psr {

struct RefineOptions {
  uint64_t bins = 128;
  uint64_t subints = 64;
  uint64_t max_evals = 40;
  double tol = 1e-3;  // stop when a step moves every parameter by < tol phase bins
  bool exact = false;  // optimise the filterbank objective itself (no cube)
  double dm_window = 0.0;  // > 0: keep DM within start +- dm_window
};

struct RefineEval {
  double J = 0.0;                        // objective
  double dP = 0.0, dPdot = 0.0, dDM = 0.0;  // gradient
  double dnu = 0.0, dnudot = 0.0;           // gradient in (1/P, -Pdot/P^2)
  double mean_y = 0.0, var_y = 0.0;      // of the dedispersed series
  std::vector<double> profile;           // B bins (sum over subints)
  std::vector<double> cells;             // S x B cloud-in-cell fold
};

// Device buffers reused across evaluations of one filterbank.
struct RefineWork {
  DevBuf dm_, dalpha_, dk_, y_, z_, parts_, cells_, g_, adj_;
  // Objective and adjoint gradient at th; v_fixed > 0 normalises J.
  int evaluate(const DeviceObs &o, uint64_t n, const psr_timing &th, const RefineOptions &opt,
               double v_fixed, RefineEval &ev, cudaStream_t st);
};

// Largest DM whose delays keep n + 1 samples inside the observation.
double max_dm_for(const DeviceObs &o, uint64_t n);

// Quasi-Newton ascent from `start`; returns the refined parameters.
int refine_gradient_one(const DeviceObs &o, uint64_t n, const psr_timing &start,
                        const RefineOptions &opt, RefineWork &w, psr_timing &out, double &J,
                        uint64_t &evals, cudaStream_t st);

// Cube buffers shared by the groups of one refinement call.
struct CubeWork;
struct CubeCache {
  CubeWork *w = nullptr;
  CubeCache() = default;
  CubeCache(const CubeCache &) = delete;
  CubeCache &operator=(const CubeCache &) = delete;
  ~CubeCache();
};

// The cube objective J at K points theta, with the cube folded at `ref`,
// and its adjoint gradient in (nu, nudot, DM) (3 values per point).
int cube_objective(const DeviceObs &o, uint64_t n, const psr_timing &ref, const psr_timing *theta,
                   uint64_t K, const RefineOptions &opt, double *J, double *grad,
                   cudaStream_t st);

// Cube-based refinement of K nearby starting points (k_refine_cube.cu).
int refine_cube_group(const DeviceObs &o, uint64_t n, const psr_timing *start, uint64_t K,
                      const RefineOptions &opt, psr_timing *out, double *J, uint64_t *evals,
                      CubeCache &cache, cudaStream_t st);

}  // namespace psr
