/*
 * ORACLE - TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the PulsarSr search path (crates fbank, rfi, dedisperse,
 * search, fold and search::confirmation), used by tests/, by the smoke check
 * and by the timed CPU baseline of bench.py.  It is the checker, never the
 * product: nothing in pulsarsr_gb300/ links or calls it.
 *
 * Parity status
 *   - fbank decode, rfi mask, dedispersion delays/plan/apply, fold, measure,
 *     window selection, grouping and the search bookkeeping are operation-by-
 *     operation restatements of the cited reference lines (f32 where Rust uses
 *     f32, f64 where Rust uses f64, sequential sums in the same order, stable
 *     sorts, total_cmp ordering, round-half-away-from-zero).  These are pinned
 *     against the reference's saved outputs (output_dm62/series.json delays,
 *     output_fold/fold.json bins and counts, the GBT RFI mask of
 *     output_confirm_gbt/report.json) and its unit-test literals.
 *   - The reference's FFT is realfft 3.5.0 / rustfft 6.4.1 (Cargo.lock), whose
 *     rounding cannot be reproduced without their source.  The oracle therefore
 *     DEFINES an FP32 real FFT (orc_raw_power: four-step + Stockham radix-16,
 *     fixed twiddle table, fmaf complex multiply) that the CUDA path reproduces
 *     bit for bit, states its error against an FP64 FFT (orc_raw_power_f64),
 *     and is pinned behaviourally against the saved schema-2 reports (family
 *     leaders, harmonic members, scores within tolerance).  Spectrum parity
 *     with rustfft itself is "unpinned at the bit level".
 */
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int64_t nchans;
  int64_t nbits;
  double tsamp;
  double fch1;
  double foff;
  int64_t data_offset;
} orc_header;

typedef struct {
  double frequency_hz;
  double period_s;
  double dm;
  uint64_t harmonics;
  double score;
} orc_candidate;

typedef struct {
  double min_hz;
  double max_hz;
  double threshold;
  uint64_t max_candidates;
  const double *birdies; /* pairs (center_hz, half_width_hz) */
  uint64_t nbirdies;
  uint64_t max_harmonics; /* 0/16: h = 1..16 as the reference; 32 adds h = 32 */
} orc_config;

typedef struct {
  double period_s;
  double snr;
  double reduced_chi_square;
} orc_profile_stats;

typedef struct {
  double snr;
  uint64_t on_samples;
  uint64_t off_samples;
  double mean_difference;
  double standard_error;
} orc_measurement;

/* Last error message of the calling thread (reference Display text). */
const char *orc_last_error(void);

int orc_parse_header(const uint8_t *bytes, uint64_t len, orc_header *out);
/* out may be NULL to query nsamples; otherwise out holds nchans*nsamples f32. */
int orc_decode(const uint8_t *bytes, uint64_t len, int64_t limit,
               orc_header *hdr, uint64_t *nsamples, float *out);

float orc_median(const float *values, uint64_t n);
int orc_channel_stats(const float *data, uint64_t nchans, uint64_t nsamples, float *means,
                      float *variances);
int orc_rfi_mask(float *data, uint64_t nchans, uint64_t nsamples,
                 uint64_t block_samples, float threshold,
                 uint64_t *channels, uint64_t *nchannels_bad,
                 uint64_t *blocks, uint64_t blocks_cap, uint64_t *nblocks_bad,
                 double *masked_fraction);

int orc_delays(const double *freqs, uint64_t nchans, double tsamp, double dm,
               uint64_t *out);
int orc_dm_step(const double *freqs, uint64_t nchans, double tsamp,
                double *out);
int orc_plan(double dm_min, double dm_max, double step, double *out,
             uint64_t cap, uint64_t *n);
int orc_apply(const float *data, uint64_t nchans, uint64_t nsamples,
              const uint64_t *delays, int64_t length, float *out,
              uint64_t *n_out);

/* The oracle's FP32 raw power spectrum (M+1 bins for N = 2*next_pow2(len)). */
int orc_raw_power(const float *series, uint64_t len, float *out);
/* FP64 reference spectrum of the same f32 input (for error statements). */
int orc_raw_power_f64(const float *series, uint64_t len, double *out);

int orc_periodicity(const float *series, uint64_t len, double tsamp, double dm,
                    const orc_config *cfg, orc_candidate *out, uint64_t cap,
                    uint64_t *n);
int orc_sift(const orc_candidate *in, uint64_t n, double resolution_hz,
             uint64_t limit, int reject_dm_zero, orc_candidate *out,
             uint64_t *n_out);

int orc_profile_at(const float *series, uint64_t n, double tsamp,
                   double period, uint64_t bins, uint64_t sample_offset,
                   orc_profile_stats *stats, float *values, uint64_t *counts);
int orc_refine(const float *series, uint64_t n, double tsamp, double frequency,
               double span_hz, uint64_t steps, uint64_t bins,
               orc_profile_stats *stats, float *values, uint64_t *counts);
int orc_measure(const float *x, uint64_t n, uint64_t offset, double tsamp,
                double period, uint64_t start_bin, uint64_t width_bins,
                uint64_t bins, orc_measurement *out);

/* The psr search trial loop: per trial delays -> apply(discovery) ->
 * periodicity, concatenated in trial order.  threads <= 0 means 1.
 * counts[i] receives the number of candidates of trial i; out holds up to
 * cap candidates in order; *n_total the full count. */
int orc_search_trials(const float *data, uint64_t nchans, uint64_t nsamples,
                      const double *freqs, double tsamp, const double *trials,
                      uint64_t ntrials, uint64_t discovery,
                      const orc_config *cfg, int threads, uint64_t *counts,
                      orc_candidate *out, uint64_t cap, uint64_t *n_total);

/* confirmation::analyze (search/src/confirmation.rs:203-496) on masked
 * channel-major data and a candidate list; malloc'd Outcome JSON (orc_free). */
char *orc_analyze_json(const float *data, uint64_t nchans, uint64_t nsamples,
                       const double *freqs, double tsamp, const double *trials,
                       uint64_t ntrials, const orc_candidate *generated,
                       uint64_t ngenerated, uint64_t limit, uint64_t bins);

/* FP64 reference of the gradient-refinement objective J and dJ/d(P, Pdot, DM)
 * (the model this project defines; no reference counterpart). */
int orc_refine_objective(const float *data, uint64_t nch, uint64_t ns,
                         const double *freqs, double tsamp, uint64_t n, double P,
                         double Pdot, double DM, uint64_t bins, uint64_t subints,
                         double variance, double *J, double *grad, double *profile);

/* Whole `psr search` (minus plots, hashing and file output) on the bytes of a
 * SIGPROC file; returns a malloc'd JSON document (free with orc_free). */
char *orc_psr_search_json(const uint8_t *bytes, uint64_t len, double dm_min,
                          double dm_max, double dm_step /* <=0: default */,
                          double min_hz, double max_hz, double threshold,
                          uint64_t top, uint64_t bins, int no_rfi,
                          const double *birdies, uint64_t nbirdies,
                          int64_t max_samples, int threads);
void orc_free(void *p);

#ifdef __cplusplus
}
#endif
