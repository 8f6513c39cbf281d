/*
 * libpsr - GB300 (sm_103a) implementation of the PulsarSr search path.
 *
 * A C ABI (plain pointers and sizes) whose functions mirror the reference's
 * crate functions one to one, so a Rust `extern "C"` block (or ctypes, cgo,
 * JNI ...) can bind them in place of the crate calls.  Each declaration cites
 * the reference function it replaces (paths inside the PulsarSr project).
 *
 * Conventions
 *   - Every function returns a status (PSR_OK == 0).  On failure the calling
 *     thread's message is available from psr_last_error(); for the error kinds
 *     that the reference reports through Display it carries the same text
 *     ("invalid or unsupported filterbank: ...", "invalid dedispersion
 *     input: ...").  Cases where the reference panics (assert!) return
 *     PSR_EINVAL.
 *   - Host buffers are allocated by the caller, with explicit capacities.
 *     Opaque handles (psr_fb, psr_session) are freed by their psr_*_free.
 *   - Arrays follow the reference layout: filterbank data is channel-major,
 *     data[channel * nsamples + time], as in fbank::Filterbank.
 *   - Handles are not shared between threads; each owns one CUDA stream.
 *     Functions are reentrant.  Everything runs on the current CUDA device.
 */
#ifndef PSR_H
#define PSR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  PSR_OK = 0,
  PSR_EIO = 1,          /* fbank::Error::Io */
  PSR_EFORMAT = 2,      /* fbank::Error::Format */
  PSR_EDEDISPERSE = 3,  /* dedisperse::Error */
  PSR_EINVAL = 4,       /* a reference assert! / invalid argument */
  PSR_ECUDA = 5,        /* CUDA runtime failure (message names the call) */
  PSR_ETIMEOUT = 6,     /* a bounded device wait gave up */
  PSR_ECAPACITY = 7     /* a caller buffer is too small (size reported) */
};

/* fbank::Header (fbank/src/lib.rs:29-38); keyword map omitted. */
typedef struct {
  int64_t nchans;
  int64_t nbits;
  double tsamp;
  double fch1;
  double foff;
  int64_t data_offset;
} psr_header;

/* search::Candidate (search/src/lib.rs:6-13). */
typedef struct {
  double frequency_hz;
  double period_s;
  double dm;
  uint64_t harmonics;
  double score;
} psr_candidate;

/* search::Config (search/src/lib.rs:14-32); birdies are (center, half width)
 * pairs, 2*nbirdies doubles.  max_harmonics is the largest harmonic sum:
 * 0 or 16 gives the reference's levels h = 1, 2, 4, 8, 16
 * (search/src/lib.rs:76); 32 adds h = 32 (an extension with no reference
 * counterpart, same score formula).  Other values are rejected. */
typedef struct {
  double min_hz;
  double max_hz;
  double threshold;
  uint64_t max_candidates;
  const double *birdies;
  uint64_t nbirdies;
  uint64_t max_harmonics;
} psr_search_config;

/* fold::Profile scalars (fold/src/lib.rs:3-11); bins/counts are arrays. */
typedef struct {
  double period_s;
  double snr;
  double reduced_chi_square;
} psr_profile_stats;

/* Spin and dispersion parameters of a refinement: period (s), period
 * derivative (s/s) and DM (pc cm^-3). */
typedef struct {
  double period_s;
  double pdot;
  double dm;
} psr_timing;

/* confirmation::Measurement (search/src/confirmation.rs:52-59). */
typedef struct {
  double snr;
  uint64_t on_samples;
  uint64_t off_samples;
  double mean_difference;
  double standard_error;
} psr_measurement;

/* Library version string ("pulsarsr-gb300 <semver> sm_103a"). */
const char *psr_version(void);
/* Copy the calling thread's last error message (NUL-terminated, truncated
 * to len).  Returns the full message length. */
uint64_t psr_last_error(char *buf, uint64_t len);

/* ------------------------------------------------------------- fbank */
/* fbank::parse_header (fbank/src/lib.rs:72-147), host. */
int psr_parse_header(const uint8_t *bytes, uint64_t len, psr_header *out);
/* The parsed fbank::Header as serde_json writes it (psr header, header.json):
 * the sorted keyword map "fields", then nchans, nbits, tsamp, fch1, foff,
 * data_offset.  *needed receives the length without the NUL; at most cap
 * bytes including the NUL are copied to buf (which may be NULL). */
int psr_header_json(const uint8_t *bytes, uint64_t len, int pretty, char *buf,
                    uint64_t cap, uint64_t *needed);

/* Device-resident filterbank: the decoded samples live in HBM, channel-major,
 * stored in their integer width (u8 for nbits <= 8, u16, or f32). */
typedef struct psr_fb psr_fb;
/* fbank::decode (fbank/src/lib.rs:149-196): header parsed on the host, the
 * packed payload copied once to the device and unpacked there. */
int psr_fb_decode(const uint8_t *bytes, uint64_t len, int64_t limit /* <0: none */,
                  psr_fb **out);
/* fbank::read (fbank/src/lib.rs:198-203): the file's payload streams to the
 * device in chunks through pinned staging buffers (reads overlap copies) and
 * is unpacked there; limit as in psr_fb_decode. */
int psr_fb_read(const char *path, int64_t limit, psr_fb **out);
int psr_fb_info(const psr_fb *fb, psr_header *header, uint64_t *nsamples);
/* A seeded synthetic filterbank generated directly on the device (the psr
 * synth command, synth/src/lib.rs:37-88, and large test shapes).  Same signal
 * model as the reference (Gaussian noise plus dispersed Gaussian pulses with
 * fractional delays), but the noise stream is a counter-based hash of
 * (seed, channel, sample), not the reference's ChaCha8 stream.  Integer bit
 * depths are rounded and clamped. */
typedef struct {
  double period_s;
  double pdot;
  double dm;
  double duty;       /* Gaussian FWHM as a fraction of the period, (0, 0.5) */
  double amplitude;  /* peak in units of the noise sigma */
  double phase;      /* pulse phase offset (cycles); the reference uses 0.25 */
} psr_synth_pulsar;
typedef struct {
  int64_t nchans;
  int64_t nbits;     /* 1, 2, 4, 8, 16 or 32 (f32) */
  uint64_t nsamples;
  double tsamp;
  double fch1;
  double foff;
  uint64_t seed;
  double noise_mean;
  double noise_sigma;
  double gain_spread;  /* per-channel gains uniform in 1 +- gain_spread */
  const psr_synth_pulsar *pulsars;
  uint64_t npulsars;   /* at most 64 */
} psr_synth_config;
int psr_fb_synth(const psr_synth_config *cfg, psr_fb **out);
/* Seeded interference added in place to a device filterbank (no reference
 * counterpart; the survey-scale workload's narrowband and burst RFI):
 * nb_channels distinct channels get nb_amplitude * (0.5 + 0.5 sin(2 pi nb_hz t
 * + phase_c)), and nbursts broadband bursts of burst_samples samples add
 * burst_amplitude to every channel; amplitudes are in sample units, integer
 * samples are rounded and clamped again. */
typedef struct {
  uint64_t seed;
  uint64_t nb_channels;
  double nb_amplitude;
  double nb_hz;
  uint64_t nbursts;      /* at most 1024 */
  uint64_t burst_samples;
  double burst_amplitude;
} psr_synth_rfi;
int psr_fb_inject_rfi(psr_fb *fb, const psr_synth_rfi *rfi);
/* Filterbank.data as f32, channel-major (nchans * nsamples values). */
int psr_fb_download(const psr_fb *fb, float *out);
/* Channels [c0, c0 + nchannels) of Filterbank.data (nchannels * nsamples
 * values): a slice of `data` without copying the rest of a large survey
 * observation to the host. */
int psr_fb_download_channels(const psr_fb *fb, uint64_t c0, uint64_t nchannels,
                             float *out);
void psr_fb_free(psr_fb *fb);

/* --------------------------------------------------------------- rfi */
/* rfi::median (rfi/src/lib.rs:4-12): upper median, exact, on the device. */
int psr_median(const float *values, uint64_t n, float *out);
/* rfi::mask (rfi/src/lib.rs:31-96) applied in place to the device samples.
 * channels has room for nchans entries; blocks for blocks_cap entries. */
int psr_rfi_mask(psr_fb *fb, uint64_t block_samples, float threshold,
                 uint64_t *channels, uint64_t *nchannels_bad, uint64_t *blocks,
                 uint64_t blocks_cap, uint64_t *nblocks_bad,
                 double *masked_fraction);
/* The per-channel means and variances that rfi::mask computes before its
 * decisions (rfi/src/lib.rs:35-43): f32 sums in the reference's order, bit
 * for bit, on the device filterbank (not modified).  nchans floats each. */
int psr_channel_stats(const psr_fb *fb, float *means, float *variances);

/* -------------------------------------------------------- dedisperse */
/* dedisperse::delays (dedisperse/src/lib.rs:9-34), host FP64, bit-exact. */
int psr_delays(const double *freqs, uint64_t nchans, double tsamp, double dm,
               uint64_t *out);
/* dedisperse::dm_step (dedisperse/src/lib.rs:35-44). */
int psr_dm_step(const double *freqs, uint64_t nchans, double tsamp, double *out);
/* dedisperse::plan (dedisperse/src/lib.rs:45-60); *n receives the trial
 * count even when cap is too small (then PSR_ECAPACITY). */
int psr_plan(double dm_min, double dm_max, double step, double *out,
             uint64_t cap, uint64_t *n);
/* dedisperse::apply (dedisperse/src/lib.rs:61-90) on a device filterbank.
 * length < 0 means the longest valid output.  out holds *n_out floats. */
int psr_dedisperse(const psr_fb *fb, const uint64_t *delays, int64_t length,
                   float *out, uint64_t cap, uint64_t *n_out);
/* Many trials at once: out is [ntrials][length] (the CLI loop,
 * cli/src/main.rs:462-469, without the periodicity step).  sums (may be
 * NULL) receives each series' f64 sum, the value periodicity's mean divides
 * (search/src/lib.rs:36): equal to the reference's sequential sum. */
int psr_dedisperse_trials(const psr_fb *fb, const double *trials,
                          uint64_t ntrials, uint64_t length, float *out,
                          double *sums);
/* Tuning, no reference counterpart: how the many-trial dedispersion of
 * psr_dedisperse_trials, searches and sessions treats samples stored in 8
 * bits (<= 8-bit data).  0: every channel added to every trial; 4 or 8:
 * channels in subbands of that width, each subband's partial sum formed once
 * per distinct intra-subband delay pattern of 8 consecutive trials and added
 * shifted to every trial that shares it (identical results); -1 (initial):
 * the library default.  Process-wide; affects searches prepared afterwards. */
int psr_set_dedisp_subbands(int subbands);

/* Test hook, no reference counterpart: one dedispersion launch (DM 0, up to
 * 8192 samples) whose staged kernel arms its TMA barriers but issues no
 * copy, so every bounded wait runs out after spin_limit polls (1..2^26) with
 * nothing in flight.  Returns PSR_ETIMEOUT with the message a real give-up
 * produces, PSR_EINVAL when the filterbank's samples do not take the staged
 * kernel (f32, or sums that could pass 2^24).  The CUDA context stays usable. */
int psr_test_stage_timeout(const psr_fb *fb, uint64_t spin_limit);

/* ------------------------------------------------------------ search */
/* The raw power spectrum of search::periodicity (search/src/lib.rs:35-44):
 * mean removal, zero padding to N = 2*next_pow2(len), real FFT, |X|^2.
 * out holds N/2 + 1 floats. */
int psr_raw_power(const float *series, uint64_t len, float *out);
/* psr_raw_power without any device allocation.  No counterpart in the
 * reference (a CPU program has no device memory to allocate).
 *
 * For callers that must not allocate device memory while they run: a process
 * whose device memory is handed out up front to another pool (a framework's
 * caching allocator, an MPS client under a memory limit), or a real-time
 * caller that cannot take the device-wide synchronisation of cudaFree while
 * other streams are busy.  psr_raw_power allocates and frees its buffers on
 * every call; this entry point computes the same spectrum, bit for bit, with
 * the same kernels, using one fixed device array of about 28 MiB reserved
 * when the library's module is loaded on a device.
 *
 *   - len must be at most PSR_RAW_POWER_NOALLOC_MAX_LEN samples; longer
 *     series return PSR_ECAPACITY (use psr_raw_power for them).
 *   - series and out are host buffers as in psr_raw_power (out: N/2 + 1
 *     floats); stream is a cudaStream_t (NULL: the default stream).  The call
 *     returns after synchronising that stream.
 *   - The first call on a device (the one current on the calling thread)
 *     looks up the array's address with cudaGetSymbolAddress; make that first
 *     call before any stream capture on the device.
 *   - Every call on a device shares the one array (series, work, spectrum and
 *     twiddle tables, which are kept between calls of the same FFT size), so
 *     calls that overlap in time on one device, from several threads or
 *     streams, race and corrupt each other's results: serialise them.
 *   - The array's address and the kept tables belong to the device's primary
 *     context (the one the CUDA runtime uses).  After cudaDeviceReset, or
 *     with another driver-API context current on that device, they are stale:
 *     do not call this entry point in either situation.
 *   - The array is reserved when the module is loaded.  With lazy module
 *     loading (CUDA_MODULE_LOADING=LAZY, the default since CUDA 12.2) that
 *     is the first call of this entry point on a device; with eager loading
 *     every process that loads libpsr holds it on every device it uses. */
#define PSR_RAW_POWER_NOALLOC_MAX_LEN (1u << 20)
int psr_raw_power_noalloc(const float *series, uint64_t len, float *out, void *stream);
/* search::periodicity (search/src/lib.rs:33-145) on one host series. */
int psr_periodicity(const float *series, uint64_t len, double tsamp, double dm,
                    const psr_search_config *cfg, psr_candidate *out,
                    uint64_t cap, uint64_t *n);
/* The psr search trial loop (cli/src/main.rs:462-473): for every trial DM,
 * delays -> apply(discovery) -> periodicity, candidates concatenated in trial
 * order.  counts[i] gets trial i's count; *n_total the total. */
int psr_search_trials(const psr_fb *fb, const double *trials, uint64_t ntrials,
                      uint64_t discovery, const psr_search_config *cfg,
                      uint64_t *counts, psr_candidate *out, uint64_t cap,
                      uint64_t *n_total);
/* search::sift (search/src/lib.rs:147-176), host. */
int psr_sift(const psr_candidate *in, uint64_t n, double resolution_hz,
             uint64_t limit, int reject_dm_zero, psr_candidate *out,
             uint64_t *n_out);

/* -------------------------------------------------------------- fold */
/* fold::profile_at (fold/src/lib.rs:16-80); values/counts hold bins entries. */
int psr_profile_at(const float *series, uint64_t n, double tsamp, double period,
                   uint64_t bins, uint64_t sample_offset,
                   psr_profile_stats *stats, float *values, uint64_t *counts);
/* fold::refine (fold/src/lib.rs:81-97): all steps+1 folds in one launch. */
int psr_refine(const float *series, uint64_t n, double tsamp, double frequency,
               double span_hz, uint64_t steps, uint64_t bins,
               psr_profile_stats *stats, float *values, uint64_t *counts);
/* confirmation::measure (search/src/confirmation.rs:107-141). */
int psr_measure(const float *x, uint64_t n, uint64_t offset, double tsamp,
                double period, uint64_t start_bin, uint64_t width_bins,
                uint64_t bins, psr_measurement *out);

/* ------------------------------------------------ gradient refinement */
/* Refinement of (P, Pdot, DM) by gradient ascent on a differentiable fold
 * objective.  No counterpart in the reference, whose refinement is the grid of
 * fold::refine (fold/src/lib.rs:81-97) plus the half-step DM grid of
 * confirmation::analyze (confirmation.rs:295-310); psr_refine_grid runs that
 * grid, and this is offered beside it.
 *
 * Objective on samples t in [0, n) of a device filterbank:
 *   y(t)  = sum_c (1-a_c) x[c][t+m_c] + a_c x[c][t+m_c+1]  with
 *           m_c + a_c = 4148.808 DM (f_c^-2 - f_max^-2) / tsamp  (fractional,
 *           linear-interpolated delays);
 *   phase = nu T + nudot T^2 / 2, T = t tsamp, nu = 1/P, nudot = -Pdot/P^2;
 *   each sample is split between its two nearest of `bins` phase bins
 *   (weights 1-w, w) and folded into `subints` equal time parts;
 *   J = sum_b (p_b - mean p)^2 / (n v), p_b summed over subints, v the
 *   variance of y (at the starting point for psr_refine_gradient).
 * The gradient comes from a hand-written adjoint; one objective + gradient
 * evaluation reads the filterbank once. */
typedef struct {
  uint64_t bins;       /* phase bins (default 128) */
  uint64_t subints;    /* time subintegrations (default 64) */
  uint64_t max_evals;  /* objective evaluations per candidate (default 40) */
  double tol_bins;     /* stop when a step moves < tol_bins phase bins (1e-3) */
  int32_t exact;       /* 0 (default): fold once per group of nearby starting
                          points into a channels x subints x bins cube at a
                          reference (P, Pdot, DM) and optimise on it, each
                          (channel, subint) profile shifted by its phase change
                          at the subint centre; 1: every evaluation runs the
                          objective above on the filterbank */
  double dm_window;    /* > 0: keep DM within start +- dm_window (the grid
                          searches +-10 half steps); 0: unbounded */
} psr_refine_options;
void psr_refine_options_default(psr_refine_options *out);
/* J and dJ/d(P, Pdot, DM) at theta.  variance <= 0 uses the variance of y at
 * theta.  profile (bins values) and subint_profiles (subints*bins) may be
 * NULL. */
int psr_refine_objective(const psr_fb *fb, uint64_t n, const psr_timing *theta,
                         const psr_refine_options *opt, double variance, double *J,
                         double *grad, double *profile, double *subint_profiles);
/* The objective psr_refine_gradient optimises by default (exact = 0): the
 * channels x subints x bins cube folded at `reference`, each (channel,
 * subint) row shifted by its phase change at the subint centre (band-limited,
 * in the Fourier domain), J = sum_b (p_b - mean p)^2 / (n v) (by Parseval,
 * from the harmonics) with v the summed channel variances; J[k] and its adjoint
 * gradient grad[3k..3k+2] = dJ/d(P, Pdot, DM) at each of npoints points
 * theta.  No reference counterpart; exposed so the fast path's adjoint can be
 * checked against finite differences and an FP64 model. */
int psr_refine_cube_objective(const psr_fb *fb, uint64_t n, const psr_timing *reference,
                              const psr_timing *theta, uint64_t npoints,
                              const psr_refine_options *opt, double *J, double *grad);
/* Gradient refinement (quasi-Newton ascent) of ncand starting points. */
int psr_refine_gradient(const psr_fb *fb, uint64_t n, const psr_timing *start,
                        uint64_t ncand, const psr_refine_options *opt,
                        psr_timing *out, double *J, uint64_t *evals);
/* The reference's grid refinement on the device, for each starting point:
 * integer-delay dedispersion at the start DM, fold::refine over 41
 * frequencies within +-resolution_hz of 1/P, then 21 DMs at half dm_step
 * around the start (clamped to [dm_lo, dm_hi]) folded at the refined period;
 * the best reduced chi-square wins.  Pdot is passed through unchanged. */
int psr_refine_grid(const psr_fb *fb, uint64_t n, const psr_timing *start,
                    uint64_t ncand, double resolution_hz, double dm_step, double dm_lo,
                    double dm_hi, uint64_t bins, psr_timing *out,
                    double *reduced_chi_square);

/* ------------------------------------------------------ confirmation */
/* confirmation::Rules (search/src/confirmation.rs:17-40); the version string
 * is always "split-confirm-v1". */
typedef struct {
  double minimum_validation_snr;
  double minimum_part_snr;
  uint64_t minimum_time_parts;
  uint64_t minimum_subbands;
  double minimum_dm_contrast;
  double minimum_dispersion_widths;
  double maximum_zero_dm_spectral_ratio;
} psr_rules;
/* Rules::default() (confirmation.rs:27-39). */
void psr_rules_default(psr_rules *out);

/* confirmation::Window (confirmation.rs:41-46). */
typedef struct {
  uint64_t start_bin;
  uint64_t width_bins;
  uint64_t bins;
} psr_window;

/* confirmation::group (confirmation.rs:177-199), host: candidates sorted by
 * score (stable, descending) and assigned to harmonic families.  order[k] is
 * the input index of the k-th candidate in score order and family[k] its
 * family (-1 when it started no family because `limit` families exist);
 * the leader of family f is the first k with family[k] == f. */
int psr_group(const psr_candidate *in, uint64_t n, double resolution_hz,
              uint64_t limit, uint64_t *order, int64_t *family,
              uint64_t *nfamilies);

/* Scalar fields of confirmation::ConfirmedCandidate (confirmation.rs:70-91).
 * rejection_mask bit i is set for reason i in the order the reference checks
 * them: 0 held-out SNR, 1 time segments, 2 subbands, 3 zero-DM control,
 * 4 dispersion sweep, 5 zero-DM spectral ratio. */
typedef struct {
  psr_candidate candidate;
  double refined_dm;
  psr_profile_stats profile;
  psr_window window;
  psr_measurement validation;
  psr_measurement zero_dm_validation;
  double zero_dm_period_s;
  psr_window zero_dm_window;
  double dm_contrast;
  double dispersion_widths;
  double zero_dm_related_spectral_ratio;
  psr_measurement time_parts[4];
  psr_measurement subbands[4];
  uint64_t harmonic_members;
  int32_t accepted;
  uint32_t rejection_mask;
} psr_confirmed;

/* confirmation::Outcome (confirmation.rs:93-101), owned by the library. */
typedef struct psr_outcome psr_outcome;
typedef struct {
  uint64_t discovery_samples;
  uint64_t validation_start_sample;
  uint64_t validation_samples;
  uint64_t common_samples;
  uint64_t trial_count;
  uint64_t candidates;
} psr_outcome_info;

/* confirmation::analyze (confirmation.rs:203-496) on a device filterbank
 * (after psr_rfi_mask where the CLI masks): the zero-DM control search,
 * harmonic families, and for each family the frequency refinement, the
 * half-step DM grid, the held-out validation, the zero-DM control, time
 * parts, subbands, per-channel discovery profiles and the DM response, all
 * computed on the device.  rules NULL means Rules::default().  Errors are the
 * reference's dedisperse::Error texts (PSR_EDEDISPERSE). */
int psr_analyze(const psr_fb *fb, const double *trials, uint64_t ntrials,
                const psr_candidate *generated, uint64_t ngenerated,
                uint64_t limit, uint64_t bins, const psr_rules *rules,
                psr_outcome **out);
int psr_outcome_info_get(const psr_outcome *o, psr_outcome_info *out);
/* Candidate i; profile_bins/profile_counts (bins entries) may be NULL. */
int psr_outcome_candidate(const psr_outcome *o, uint64_t i, psr_confirmed *out,
                          float *profile_bins, uint64_t *profile_counts);
/* The Outcome as serde_json writes it (field order and number format of the
 * reference), compact or pretty.  Copies at most len bytes including the
 * NUL; returns the full length without the NUL. */
uint64_t psr_outcome_json(const psr_outcome *o, int pretty, char *buf,
                          uint64_t len);
void psr_outcome_free(psr_outcome *o);

/* ----------------------------------------------------------- session */
/* A whole search of one observation shape kept resident on the device:
 * packed payload -> unpack -> RFI mask -> trial loop -> per-trial candidate
 * lists.  Buffers are allocated once at creation, so run() allocates
 * nothing; this is the call a survey pipeline repeats per observation.
 * rfi_block_samples == 0 disables masking (psr search --no-rfi). */
typedef struct psr_session psr_session;
int psr_session_create(const psr_header *header, uint64_t nsamples,
                       const double *trials, uint64_t ntrials,
                       uint64_t discovery, const psr_search_config *cfg,
                       uint64_t rfi_block_samples, float rfi_threshold,
                       psr_session **out);
/* Copy a packed payload (the bytes after the header) from host memory. */
int psr_session_load(psr_session *s, const uint8_t *payload, uint64_t nbytes);
/* Enqueue unpack + mask + search on the session stream (asynchronous). */
int psr_session_run(psr_session *s);
/* Wait for the session stream; reports device-side errors. */
int psr_session_sync(psr_session *s);
/* Results of the last run (after sync). */
int psr_session_candidates(psr_session *s, uint64_t *counts, psr_candidate *out,
                           uint64_t cap, uint64_t *n_total);
int psr_session_mask(psr_session *s, uint64_t *channels, uint64_t *nchannels_bad,
                     uint64_t *blocks, uint64_t blocks_cap, uint64_t *nblocks_bad,
                     double *masked_fraction);
/* Diagnostics with no counterpart in the reference (which only times whole
 * runs, cli/src/main.rs:415): when enabled, run() records CUDA events around
 * every stage on the session stream.  enable 1: the stages overlap as in an
 * unprofiled run (the spectrum stage of a chunk beside the next chunk's
 * dedispersion and FFT); 2: serialised, each chunk's dedispersion waits for
 * the previous chunk's spectrum stage, so each stage's time is its own
 * kernels' alone.  stage_times() fills ms[5] and launches[5] for (unpack,
 * rfi, dedisperse, fft, spectrum), summed over the runs since the last
 * reset. */
int psr_session_set_profiling(psr_session *s, int enable);
int psr_session_stage_times(psr_session *s, double *ms, uint64_t *launches, int reset);
/* confirmation::analyze over the last run's candidates (the psr search
 * command, cli/src/main.rs:474-478), on the session's masked observation. */
int psr_session_analyze(psr_session *s, uint64_t limit, uint64_t bins,
                        const psr_rules *rules, psr_outcome **out);
/* ------------------------------------------------------------- batch */
/* Many observations of uneven shape (channels, length, DM plan) searched by
 * one CUDA graph launch (the examples' serial observation loops,
 * cli/src/main.rs:462-473 per observation).  No reference counterpart for the
 * batching itself.  Each observation keeps its own session; psr_batch_run
 * captures all of them, concurrently, into one graph on first use and
 * launches that graph afterwards.  hbm_budget_bytes bounds the dedispersed
 * series and spectra held at once (0: 64 GiB): it sets the trials per
 * dedispersion block. */
typedef struct {
  psr_header header;
  uint64_t nsamples;
  const double *trials;
  uint64_t ntrials;
  uint64_t discovery;
  psr_search_config config;
  uint64_t rfi_block_samples;
  float rfi_threshold;
} psr_batch_obs;
typedef struct psr_batch psr_batch;
int psr_batch_create(const psr_batch_obs *obs, uint64_t n, uint64_t hbm_budget_bytes,
                     psr_batch **out);
int psr_batch_load(psr_batch *b, uint64_t i, const uint8_t *payload, uint64_t nbytes);
/* Load observation i from an 8-bit device filterbank of the same shape (its
 * samples packed into the time-major payload on the device). */
int psr_batch_load_fb(psr_batch *b, uint64_t i, const psr_fb *fb);
/* Autotuner: per shape class (channels, bit depth, FFT size, trial count to
 * the nearest power of two), times whole searches of the class's first
 * loaded observation at each candidate tiling (DM block and half of it;
 * whole-block or 64-trial FFT launches; for 8-bit samples, channel-by-channel
 * or 8-channel subband dedispersion) and applies the fastest to the class.
 * chunk/inner/subbands (n entries each, may be NULL) receive the choices. */
int psr_batch_tune(psr_batch *b, uint64_t *chunk, uint64_t *inner, int *subbands);
/* Pin observation i's dedispersion block (trials per outer chunk, >= 1) and
 * FFT launch size (trials per inner chunk; 0 = the whole block within a 4 GB
 * work buffer): the manual counterpart of psr_batch_tune.  No reference
 * counterpart. */
int psr_batch_set_chunking(psr_batch *b, uint64_t i, uint64_t chunk, uint64_t inner);
int psr_batch_run(psr_batch *b);
int psr_batch_sync(psr_batch *b);
int psr_batch_candidates(psr_batch *b, uint64_t i, uint64_t *counts, psr_candidate *out,
                         uint64_t cap, uint64_t *n_total);
void *psr_batch_stream(psr_batch *b);
void psr_batch_free(psr_batch *b);

/* Device copy of the packed payload buffer (for device-resident timing). */
void *psr_session_payload_device(psr_session *s);
/* The session's CUDA stream (cudaStream_t), for event timing. */
void *psr_session_stream(psr_session *s);
void psr_session_free(psr_session *s);

#ifdef __cplusplus
}
#endif
#endif /* PSR_H */
