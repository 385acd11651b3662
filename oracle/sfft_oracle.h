/*
 * sfft_oracle.h — CPU restatement of the sFFT 0.1 exec path (v1/v2/v3).
 *
 * TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py use it, as the checker.  The
 * product (sfft_gb300/) never links or calls it.
 *
 * Every function follows the reference file:line cited at its definition
 * in sfft_oracle.c.  Randomness comes from glibc random() / drand48() in
 * the reference's draw order, so seeding with srandom(s); srand48(s)
 * before an exec reproduces the reference's permutations.
 */
#ifndef SFFT_ORACLE_H
#define SFFT_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_plan oracle_plan;

/* Plan fields as in src/sfft.h:81-154 (what the reference computes). */
typedef struct
{
  int version;                  /* 0 = v1, 1 = v2, 2 = v3 (src/sfft.h:37-42) */
  int n, k;                     /* n already floored to a power of two */
  /* v1 / v2 */
  int B_loc, B_thresh, B_est, W_Comb, Comb_loops;
  int loops_loc, loops_thresh, loops_est;
  int w_loc, w_est;
  long x_samp_size;
  /* v3 */
  int B_g1, w_g1, B_g2, w_g2, W_Man;
  int Gauss_loops, Gauss2_loops, Man_loops;
} oracle_params;

oracle_plan *oracle_make_plan(int n, int k, int version);
void oracle_get_params(const oracle_plan *p, oracle_params *out);
/* which: 0 = location / first Gaussian filter, 1 = estimation / second.
 * time: 2*w doubles; freq: 2*n doubles (interleaved re, im). */
const double *oracle_filter_time(const oracle_plan *p, int which);
const double *oracle_filter_freq(const oracle_plan *p, int which);
void oracle_free_plan(oracle_plan *p);

/* One transform of the 2n-double signal `in`.  Writes the recovered
 * coefficients sorted by frequency (distinct frequencies; v1/v2 values are
 * the reference's, i.e. conjugated, src/computefourier-1.0-2.0.cc:383-398).
 * Returns the number of entries, or -1 if cap is too small / bad input. */
long oracle_exec(oracle_plan *p, const double *in, int *out_idx,
                 double *out_val, long cap);

/* As oracle_exec for `num` signals, OpenMP-parallel over signals like
 * sfft_exec_many (src/sfft.cc:139-147); writes dense n-point outputs. */
void oracle_exec_many_dense(oracle_plan *p, int num, const double **in,
                            double **out);

/* Debug views of thread 0's last exec (valid until the next exec). */
const int *oracle_dbg_perm(const oracle_plan *p, int which); /* 0 a, 1 ai */
const int *oracle_dbg_J(const oracle_plan *p);       /* loops * B_thresh */
const int *oracle_dbg_score(const oracle_plan *p);   /* n vote counts */
const int *oracle_dbg_hits(const oracle_plan *p, long *count);
const double *oracle_dbg_xsamp(const oracle_plan *p);        /* buckets */
const int *oracle_dbg_comb(const oracle_plan *p, int *count);
/* v3: a, ai, b, init_offset, init_G_offset, passes, early_exit, n_found */
void oracle_dbg_v3(const oracle_plan *p, int *vals);
/* v3: every tone estimate of the last exec as (round, stage, key, re, im);
 * round -2 is the first comb pass, -1 the first Gaussian pass, then the
 * round-robin loop.  Returns the number of records. */
long oracle_dbg_v3_trace(const oracle_plan *p, double *out, long cap);

#ifdef __cplusplus
}
#endif

#endif
