// Search engine shared by the C ABI entry points and the session.
#pragma once
#include "psr_internal.h"

namespace psr {

struct SearchEngine {
  // Trials per outer chunk (dedispersion and candidate selection run over
  // the whole chunk) and per inner chunk (FFT and normalisation launches;
  // large launches amortise their tails, so by default the whole chunk
  // within a 4 GB FFT work buffer).  0 = automatic.
  uint64_t chunk = 0;
  uint64_t inner = 0;
  // Dedispersion subband width for 8-bit-storage samples: 0 = channel by
  // channel, 4 or 8 = subband reuse, -1 = the library default
  // (dedisp_subbands_default()).
  int subbands = -1;
  SubbandPlan sbplan;
  uint64_t ntrials = 0, n = 0, nch = 0, ldo = 0, ldp = 0, nparts = 0, nchunks = 0;
  // Outer chunk ci covers trials [cstart[ci], cstart[ci + 1]).  A search of
  // more than one chunk ends with a short chunk (chunk / 8 trials): the
  // spectrum stage of the last chunk has nothing left to overlap with.
  std::vector<uint64_t> cstart;
  uint64_t max_spread = 0;
  uint32_t npsum = 0;
  FftPlan fft;
  SpecConfig spec;
  SpecWork sw;
  // Optional per-stage timing: events recorded around every stage launch on
  // the engine's stream; stage_ms accumulates their elapsed times.  profile
  // 1: stages overlap as in an untimed run; 2: serialised, each chunk's
  // dedispersion waits for the previous chunk's spectrum work, so every
  // stage's time is its kernels' own (no SMs shared with the other stream).
  enum { ST_DEDISP = 0, ST_FFT = 1, ST_SPEC = 2, ST_COUNT = 3 };
  int profile = 0;
  std::vector<cudaEvent_t> ev_begin[ST_COUNT], ev_end[ST_COUNT];
  double stage_ms[ST_COUNT] = {0, 0, 0};
  uint64_t stage_launches[ST_COUNT] = {0, 0, 0};
  int record(int stage, bool begin, cudaStream_t st);
  int harvest();  // after a sync: add elapsed times, forget the events
  ~SearchEngine();
  DevBuf delays, trial_dm, series, parts, sums, means, work, power, psum, kept, kept_count, err,
      chunk_overflow;
  HostBuf h_kept, h_kept_count;  // collect()'s staging of the kept lists
  HostBuf h_status;              // finish(): overflow and error words
  // The gates, harmonic items and selection of a chunk run on `aux`, so that
  // they overlap the FFTs of the following inner chunks and of the next
  // chunk on the caller's stream.  ev_fft[i % 2]: FFT of inner chunk i done.
  // The power spectra and their partial sums are double-buffered by chunk
  // parity: ev_sel[b] = selection of the last chunk in half b done.
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fft[2] = {nullptr, nullptr}, ev_sel[2] = {nullptr, nullptr};
  bool sel_pending[2] = {false, false};

  // Delay tables, FFT plan and buffers for ntrials trials of length n.
  int prepare(const DeviceObs &o, const double *trials, uint64_t ntrials, uint64_t n,
              const SpecConfig &cfg, cudaStream_t st);
  int enqueue_chunk(const DeviceObs &o, uint64_t ci, cudaStream_t st);
  // All chunks, asynchronously (joined back into st).
  int enqueue(const DeviceObs &o, cudaStream_t st);
  // Make st wait for the aux-stream work queued so far.
  int join(cudaStream_t st);
  // Synchronise; redo chunks whose raw candidate storage overflowed.
  int finish(const DeviceObs &o, cudaStream_t st);
  int collect(cudaStream_t st, uint64_t *counts, psr_candidate *out, uint64_t cap,
              uint64_t *n_total);
};

}  // namespace psr
