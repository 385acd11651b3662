/*
 * sfft.h — GB300 sparse FFT engine, drop-in C interface of sFFT 0.1.
 *
 * The first block keeps the reference's types and six exported functions
 * (sFFT 0.1 src/sfft.h:34-50 and :158-167) with the same names, layouts,
 * argument meanings and ownership rules; a program or binding written for
 * libsfft.so of sFFT 0.1 links against this library unchanged.  The second
 * block adds entry points for device-resident, batched, sparse and
 * reduced-precision use.  All entry points are extern "C", take plain
 * pointers and sizes, and never abort: failures return NULL / a negative
 * status and leave a message for sfft_last_error().
 */
#ifndef SFFT_GB300_SFFT_H
#define SFFT_GB300_SFFT_H

#include <stddef.h>

#ifdef __cplusplus
#include <unordered_map>
#endif

/* complex_t: C99 double complex, as sFFT 0.1 src/fft.h:42-45 (g++ accepts
 * the _Complex keyword as an extension, as the reference relies on). */
#ifndef SFFT_COMPLEX_T_DEFINED
#define SFFT_COMPLEX_T_DEFINED
typedef double _Complex complex_t;
#endif

/* FFTW planner flags accepted (and, as in the reference, not needed) by
 * sfft_make_plan; values of fftw3.h, which the reference binding hard-codes
 * (python/sfft/sfft.py:7-8). */
#ifndef FFTW_ESTIMATE
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
#endif

#ifdef __cplusplus
/* sFFT 0.1 src/sfft.h:34-35 (the reference used std::tr1::unordered_map). */
typedef std::unordered_map<int, complex_t> sfft_output;
#endif

/* sFFT 0.1 src/sfft.h:37-42 */
enum sfft_version
{
  SFFT_VERSION_1,
  SFFT_VERSION_2,
  SFFT_VERSION_3
};

/* sFFT 0.1 src/sfft.h:44-50.  `data` is opaque here (device-resident plan). */
struct sfft_plan
{
  enum sfft_version version;
  unsigned int n;
  unsigned int k;
  void *data;
};
typedef struct sfft_plan sfft_plan;

#ifdef __cplusplus
extern "C" {
#endif

/* ---- the reference's API (sFFT 0.1 src/sfft.h:158-167) ------------------ */

/* src/sfft.cc:60-63.  16-byte aligned; here page-locked host memory, so
 * transfers to the GPU run at full link speed.  Free with sfft_free. */
void *sfft_malloc(size_t s);
/* src/sfft.cc:65-69 */
void sfft_free(void *p);

/* src/sfft.cc:71-101.  n must be a power of two (the reference floors n
 * inside the plan but not in sfft_exec).  Returns NULL for an unknown
 * version, for (n, k) outside the algorithm's domain (v1/v2: every bucket
 * count >= 2k+1; v3: k >= 8) or when no CUDA device is usable. */
sfft_plan *sfft_make_plan(int n, int k, enum sfft_version version, int fftw_optimization);
/* src/sfft.cc:103-117 (frees everything, including the plan itself). */
void sfft_free_plan(sfft_plan *plan);
/* src/sfft.cc:119-137.  in: n complex values; out: n complex values, fully
 * overwritten (zeros except the recovered coefficients).  Either may be a
 * host or a device pointer.  v1/v2 values are those of the reference, i.e.
 * the complex conjugates of the spectrum (src/computefourier-1.0-2.0.cc:
 * 383-398).  Randomness: glibc random()/drand48(), drawn in the reference's
 * order. */
void sfft_exec(sfft_plan *plan, complex_t *in, complex_t *out);
/* src/sfft.cc:139-147.  `num` transforms with one plan, batched on the
 * GPU; draws happen in signal order. */
void sfft_exec_many(sfft_plan *plan, int num, complex_t **in, complex_t **out);

/* ---- additions (no counterpart in the reference) ------------------------ */

enum sfft_precision
{
  SFFT_PREC_FP64 = 0,           /* parity form: bit-exact v1/v2 */
  SFFT_PREC_FP32 = 1            /* fold, bucket FFTs, estimation in FP32 */
};

enum sfft_input_type
{
  SFFT_IN_C128 = 0,             /* complex128 (complex_t) */
  SFFT_IN_C64 = 1               /* complex64 (float pairs) */
};

struct sfft_options
{
  int precision;                /* enum sfft_precision */
  int device;                   /* CUDA device ordinal, -1 = current */
  int max_batch;                /* signals per launch (0 = default 16) */
};
typedef struct sfft_options sfft_options;

/* As sfft_make_plan with options (NULL = FP64, current device). */
sfft_plan *sfft_make_plan_ex(int n, int k, enum sfft_version version, int fftw_optimization,
                             const sfft_options *opt);

/* Constants of a v1/v2 plan: what the reference reads from its parameter
 * tables (src/parameters.cc).  Plans made from them are not the
 * reference's plans unless the values equal the table's. */
struct sfft_params
{
  double Bcst_loc, Bcst_est, Comb_cst;
  int loc_loops, est_loops, threshold_loops, comb_loops;
  double tolerance_loc, tolerance_est;
};
typedef struct sfft_params sfft_params;

/* A v1/v2 plan with explicit constants (params == NULL: the reference's). */
sfft_plan *sfft_make_plan_params(int n, int k, enum sfft_version version, const sfft_params *params,
                                 const sfft_options *opt);

/* The plan's own CUDA stream (a cudaStream_t): work submitted with a NULL
 * stream runs there. */
void *sfft_plan_stream(const sfft_plan *plan);

/* Device memory a plan holds (constants and workspace), in bytes. */
long sfft_plan_footprint(const sfft_plan *plan);

/* Message of the last failure on this thread ("" if none). */
const char *sfft_last_error(void);

/* Number of coefficients one transform can return (sizes sparse outputs). */
long sfft_output_capacity(const sfft_plan *plan);

/* One transform with a sparse result: writes up to `cap` (index, value)
 * pairs (host or device buffers) and returns their number, or -1. */
long sfft_exec_sparse(sfft_plan *plan, const complex_t *in, int *out_idx, complex_t *out_val,
                      long cap);

/* Batched, device-resident, asynchronous.  in: host array of `num` device
 * pointers to signals of type `in_type`.  Outputs are device buffers:
 * out_idx[s * out_stride + i], out_val likewise (complex128 for FP64 plans,
 * complex64 for FP32 plans), out_count[s].  `stream` is a cudaStream_t
 * (NULL = the plan's stream).  Returns 0 or -1. */
int sfft_exec_batch(sfft_plan *plan, int num, const void *const *in, int in_type, int *out_idx,
                    void *out_val, int *out_count, long out_stride, void *stream);

/* sfft_exec_many (src/sfft.h:167) with sparse results instead of dense
 * n-point arrays: in[s] host or device complex128 signals; out_idx[s *
 * out_stride + i] and out_val likewise (complex128 for FP64 plans,
 * complex64 for FP32 v1/v2 plans), out_count[s] -- host or device buffers
 * (page-locked host memory, e.g. from sfft_malloc, makes the copies
 * asynchronous).  Input copies, transforms and result copies of successive
 * chunks overlap.  Synchronous; returns 0, or -1 with sfft_last_error(). */
int sfft_exec_many_sparse(sfft_plan *plan, int num, const complex_t *const *in, int *out_idx, void *out_val,
                          int *out_count, long out_stride);

/* As sfft_exec_batch, with the random draws of signal s taken from
 * private generators seeded with seeds[s] exactly as srandom(seeds[s]);
 * srand48(seeds[s]) would seed the reference's (seeds == NULL: the global
 * glibc streams).  A signal's result then does not depend on the batch it
 * runs in. */
int sfft_exec_batch_ex(sfft_plan *plan, int num, const void *const *in, int in_type, const unsigned *seeds,
                       int *out_idx, void *out_val, int *out_count, long out_stride, void *stream);

/* Waits for the plan's work and reports device-side errors: 0 or -1. */
int sfft_sync(sfft_plan *plan);

/* Diagnostics of the last transform of batch slot 0, for parity checks.
 * what: 0 permutations a[L] then ai[L] (int); 1 selected buckets J[L][2k]
 * (int); 2 vote counts (n int); 3 bucket values x_samp (complex, plan
 * precision); 4 v2 comb residues (int, count returned); 5 v3 rounds;
 * 6 v3 estimates as (round, stage, frequency, re, im) doubles;
 * 7 the 16 counters of slot 0 (0 hits, 1 comb residues, 2 outputs, 3 error
 * bits, 4 frequencies that reached the vote threshold (v1 and voted v2),
 * 8 FP64 medians that took the all-exact path); 8 / 9 the
 * v1/v2 estimation window of the location / estimation filter as held on
 * the device (FP64 plans: n/B entries of (c, d, c^2 + d^2, 0) doubles, the
 * filter.freq values estimate_values divides by; FP32 plans: n/B
 * (re, im) floats of conj(h) / |h|^2).
 * Returns the number of elements written, or -1. */
long sfft_debug_fetch(sfft_plan *plan, int what, void *dst, long cap);

/* The selection network the estimators use for the lower median of n
 * values (n = 8..24, the loop counts whose networks are compiled): writes
 * (i, j, kind) per comparator in execution order -- kind 1 sets v[i] =
 * min, v[j] = max; 2 only v[i] = min(v[i], v[j]); 3 only v[j] =
 * max(v[i], v[j]) -- after which v[(n - 1) / 2] is the lower median.
 * Host only; returns the comparator count, or -1 (unsupported n, or cap
 * below 3 ints per comparator). */
int sfft_debug_median_network(int n, int *dst, long cap);

/* Stage timing with CUDA events recorded on the launching stream.
 * sfft_profile(plan, 1) starts (and zeroes) it; sfft_profile_read waits for
 * the recorded launches and writes the summed milliseconds per stage
 * (v1/v2: 0 comb filter, 1 permuted-filter fold, 2 bucket FFT + top-k
 * selection + voting, 3 median estimation; v3: 0 filters, 1 peeling);
 * it returns the number of timed launches, or -1. */
int sfft_profile(sfft_plan *plan, int enable);
long sfft_profile_read(sfft_plan *plan, double *stage_ms, int nstage);
/* Number of GPU kernels this library has launched in this process. */
long sfft_kernel_launches(void);

/* sfft_exec_noalloc has no counterpart in the reference.  One v1/v2
 * transform that allocates no GPU memory, for callers that cannot call
 * cudaMalloc while they run (memory handed to their own pool, a fixed
 * budget after start-up, or a latency-bound stream that must not be
 * synchronised by cudaMalloc/cudaFree).  Its scratch is a static 4 MiB
 * device array in this library (held on every GPU that loads it), so plans
 * are limited to n <= 2^18, at most 65536 bucket samples and 32 loops;
 * larger plans return -1.  d_in: device signal of type in_type; outputs:
 * device buffers of at least sfft_output_capacity(plan) entries
 * (complex128 values for FP64 plans, complex64 for FP32 plans);
 * d_status: device int[2] receiving the coefficient count and the device
 * error bits.  Asynchronous on `stream` (a cudaStream_t).  The first call
 * on a device looks up the static array and should precede any stream
 * capture; all calls share the array, so calls whose GPU work overlaps
 * race.  Returns 0, or -1 with sfft_last_error() set. */
long sfft_exec_noalloc(sfft_plan *plan, const void *d_in, int in_type, int *d_out_idx, void *d_out_val,
                       long cap, int *d_status, void *stream);

/* ---- serving: continuous batching on one GPU ---------------------------- */

typedef struct sfft_server sfft_server;
struct sfft_server_options
{
  int device;                   /* CUDA device, -1 = current */
  int max_batch;                /* transforms per batch of one plan (0: 32) */
  long hbm_budget_bytes;        /* device memory for plans + batches (0: 80% of free) */
  int k_round;                  /* 1: round k up to the grid ceil(8 * 2^(j/4)); 2: to a power of two */
  int tune_invalid;             /* v1/v2: 1 shapes outside the reference's domain get tuned constants;
                                   2 every v1/v2 request uses autotuned constants, k rounded to its bucket;
                                   1 and 2: v3 requests with k < 8 run on the smallest v3 plan (k = 8) */
  int v2_voted;                 /* 1: v2 plans in the voted mode (sfft_plan_v2_voted) */
};
typedef struct sfft_server_options sfft_server_options;

sfft_server *sfft_server_create(const sfft_server_options *opt);
void sfft_server_destroy(sfft_server *s);
/* Queues one transform of `in` (device or host, kept alive by the caller
 * until the request completes); returns its id, or -1. */
long sfft_server_submit(sfft_server *s, int n, int k, enum sfft_version version, int precision, const void *in,
                        int in_type, unsigned seed);
/* Waits for request `id`; writes its coefficients (host or device buffers,
 * values as complex128) and the submit-to-completion latency.  Returns the
 * number of coefficients, or -1. */
long sfft_server_wait(sfft_server *s, long id, int *out_idx, complex_t *out_val, long cap, double *latency_ms);
/* The number of coefficients of a finished request (waiting up to
 * timeout_ms, < 0: no limit; -2 on time-out), without collecting it: size
 * the buffers of sfft_server_wait with it. */
long sfft_server_count(sfft_server *s, long id, double timeout_ms);
/* As sfft_server_wait, giving up after timeout_ms (< 0: no limit): then
 * returns -2 and the request stays pending. */
long sfft_server_wait_for(sfft_server *s, long id, int *out_idx, complex_t *out_val, long cap, double *latency_ms,
                          double timeout_ms);
/* Device bytes the server reserves for a plan of this shape with
 * `max_batch` slots (its admission estimate), or -1. */
long sfft_server_plan_bytes(int n, int k, enum sfft_version version, int precision, int max_batch);
/* batches, plans made, plans evicted, deferrals, cached plans, bytes held,
 * budget, queued requests, batches whose results were moved to host memory
 * (finished, not yet collected, and their device memory needed). */
int sfft_server_stats(sfft_server *s, long *stats, int nstats);

/* ---- signals of different shapes in one CUDA graph ---------------------- */

/* sfft_exec_many for `num` signals whose (n[i], k[i], version[i],
 * precision[i]) may all differ (precision may be NULL: FP64).  Signals of
 * one plan share it and run batched; all groups run concurrently as
 * branches of one CUDA graph that later calls replay.  tune (v1/v2 only):
 * 0 the reference's constants; 1 those, else tuned constants for shapes
 * outside the reference's domain; 2 autotuned constants per (n, k bucket),
 * k rounded up to its bucket (sfft_tuned_k) so that nearby k share a plan. */
typedef struct sfft_mixed sfft_mixed;
sfft_mixed *sfft_mixed_create(int num, const int *n, const int *k, const int *version, const int *precision,
                              int in_type, int tune, int device);
/* One execution: in[i] device pointers; seeds (or NULL) as in
 * sfft_exec_batch_ex.  Asynchronous; sfft_mixed_sync waits. */
int sfft_mixed_exec(sfft_mixed *m, const void *const *in, const unsigned *seeds);
/* Waits for the last execution; -1 (message in sfft_last_error()) if a
 * kernel flagged one of its signals. */
int sfft_mixed_sync(sfft_mixed *m);
/* Device pointers to signal s's result (indices, values of value_bytes =
 * 16 (complex128) or 8 (complex64) each, capacity); returns its count. */
int sfft_mixed_result(sfft_mixed *m, int s, const int **idx, const void **val, int *value_bytes, long *cap);
/* The same copied to host memory (at most cap entries; values as above).
 * Returns the signal's count, or -1. */
long sfft_mixed_result_host(sfft_mixed *m, int s, int *idx, void *val, long cap);
int sfft_mixed_groups(const sfft_mixed *m);
/* Before the first sfft_mixed_exec: run every plain FP32 v2 group whose
 * FFTs fit in shared memory with one persistent kernel instead of one
 * branch of kernels per group -- a device work queue of (stage, plan,
 * signal, tile) items in dependency order with per-signal completion
 * counters and bounded waits.  Other groups keep their branches in the same
 * graph.  Returns 0, or -1 with sfft_last_error(). */
int sfft_mixed_set_persistent(sfft_mixed *m, int on);
/* The stream (cudaStream_t) the batch's graph runs on. */
void *sfft_mixed_stream(const sfft_mixed *m);
void sfft_mixed_destroy(sfft_mixed *m);

/* ---- v2 voted mode (no counterpart in the reference) ------------------ */

/* on = 1: the v2 plan estimates only the candidates that reached the vote
 * threshold (as v1 does) instead of every comb candidate, which the
 * reference estimates and returns (most of them noise).  The recovered
 * tones are the same; the result is not the reference's output list.
 * Call between executions; the output capacity may change.  0 or -1. */
int sfft_plan_v2_voted(sfft_plan *plan, int on);

/* ---- constants chosen by this project (no counterpart in the reference) */

/* v1/v2 constants for (n, k): the autotuner's table row for n and the k
 * bucket of k (returns 1), else a rule (returns 0); -1 if neither applies. */
int sfft_tuned_params(int n, int k, int version, sfft_params *params);
/* The k bucket: the next power of two >= max(k, 16). */
int sfft_tuned_k(int k);

/* Host-only plan queries (no GPU needed): the parameters a plan for
 * (n, k, version) would use, as the reference computes them.  fields:
 * v1/v2: B_loc, B_thresh, B_est, W_Comb, Comb_loops, loops_loc,
 * loops_thresh, loops_est, w_loc, w_est, x_samp_size; v3: W_Man, B_g1,
 * w_g1, B_g2, w_g2.  Returns the number of fields written, or -1. */
int sfft_describe_plan(int n, int k, enum sfft_version version, long *fields, int nfields);
/* The same for a v1/v2 plan with explicit constants (no counterpart in the
 * reference). */
int sfft_describe_plan_params(int n, int k, enum sfft_version version, const sfft_params *params, long *fields,
                              int nfields);
/* The filter a plan would use: which 0 = location / first Gaussian,
 * 1 = estimation / second Gaussian; time taps (2*w doubles) and the
 * n-point spectrum (2*n doubles, may be NULL).  Returns w, or -1. */
int sfft_describe_filter(int n, int k, enum sfft_version version, int which, double *time, long time_cap,
                         double *freq, long freq_cap);

#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
/* The form the sFFT documentation gives (doc/usage.rst:77): a map from
 * frequency to coefficient, filled through sfft_exec_sparse. */
#include <vector>
inline int sfft_exec_output(sfft_plan *plan, const complex_t *in, sfft_output *out)
{
  long cap = sfft_output_capacity(plan);
  if (cap < 0)
    return -1;
  std::vector<int> idx((size_t)cap);
  std::vector<complex_t> val((size_t)cap);
  long c = sfft_exec_sparse(plan, in, idx.data(), val.data(), cap);
  if (c < 0)
    return -1;
  out->clear();
  for (long i = 0; i < c; i++)
    (*out)[idx[(size_t)i]] = val[(size_t)i];
  return 0;
}
#endif

#endif
