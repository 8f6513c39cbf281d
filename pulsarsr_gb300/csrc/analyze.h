// confirmation::analyze on the device: shared by the C ABI entry points.
#pragma once
#include <string>
#include <vector>

#include "json_writer.h"
#include "psr_internal.h"

namespace psr {

// fold::Profile (fold/src/lib.rs:3-11).
struct FoldedProfile {
  psr_profile_stats st{};
  std::vector<float> values;
  std::vector<uint64_t> counts;
};

// confirmation::DmPoint (confirmation.rs:60-69).
struct DmPoint {
  double dm = 0.0;
  bool matched = false;
  double spectral_score = 0.0;
  double spectral_frequency_hz = 0.0;
  double discovery_profile_response = 0.0;
};

// confirmation::ConfirmedCandidate (confirmation.rs:70-91).
struct Confirmed {
  psr_confirmed s{};
  FoldedProfile profile;
  std::vector<float> time_profiles[4];
  std::vector<float> subband_profiles[4];
  std::vector<DmPoint> dm_response;
  std::vector<psr_candidate> members;
  std::vector<std::string> reasons;
};

// confirmation::Outcome (confirmation.rs:93-101).
struct Outcome {
  psr_rules rules{};
  psr_outcome_info info{};
  std::vector<Confirmed> candidates;
};

// confirmation::group (confirmation.rs:177-199).
struct Family {
  psr_candidate leader;
  std::vector<psr_candidate> members;
};
std::vector<Family> group_candidates(const psr_candidate *c, uint64_t n, double resolution,
                                     uint64_t limit, std::vector<uint64_t> *order = nullptr,
                                     std::vector<int64_t> *family = nullptr);

// confirmation::analyze (confirmation.rs:203-496) on a device observation.
int analyze_obs(const DeviceObs &o, const double *trials, uint64_t ntrials,
                const psr_candidate *generated, uint64_t ngenerated, uint64_t limit,
                uint64_t bins, const psr_rules &rules, Outcome &out, cudaStream_t st);

// The reference's grid refinement (fold::refine over 41 frequencies, then 21
// half-step DMs) at one starting point, on the device.
int grid_refine_one(const DeviceObs &o, uint64_t n, const psr_timing &start,
                    double resolution, double dm_step, double dm_lo, double dm_hi,
                    uint64_t bins, psr_timing &out, double &rcs, cudaStream_t st);

psrjson::Value candidate_json(const psr_candidate &c);
psrjson::Value outcome_json(const Outcome &o);

}  // namespace psr

struct psr_outcome {
  psr::Outcome o;
};
