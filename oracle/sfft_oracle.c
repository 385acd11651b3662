/*
 * sfft_oracle.c — CPU restatement of the sFFT 0.1 plan + exec path.
 *
 * TEST INFRASTRUCTURE, not product code: tests/, __graft_entry__.smoke()
 * and bench.py's CPU legs use it as the checker.  Each function cites the
 * reference file:line whose algorithm it restates (paths relative to the
 * sFFT 0.1 source tree).  Differences from the reference, on purpose:
 *   - The v3 result map iterates in insertion order (the reference's
 *     std::tr1::unordered_map order depends on its hash buckets).  This
 *     only changes the order in which peeled tones are subtracted from a
 *     bucket, i.e. rounding at the 1e-16 level.
 *   - v3 allocates w_g2 + 1 permuted samples (the reference allocates w_g2
 *     and writes w_g2 + 1, src/sfft.cc:497 vs src/computefourier-3.0.cc:235)
 *     and bounds the peeling loop (the reference loops until a fixpoint).
 *   - No SSE: the SSE expressions are written out as the scalar operations
 *     they perform, in the same order.  Build with -ffp-contract=off.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "fftw3.h"
#include "sfft_oracle.h"

#define MINI(a, b) ((a) < (b) ? (a) : (b))
#define MAXI(a, b) ((a) > (b) ? (a) : (b))
#define V3_MAX_PASSES 3000

/* ---------------------------------------------------------------- utils -- */

/* src/utils.cc:41-46 */
static int o_gcd(int a, int b)
{
  if (a % b == 0)
    return b;
  return o_gcd(b, a % b);
}

/* src/utils.cc:85-101 */
static int o_mod_inverse(int a, int n)
{
  int i = n, v = 0, d = 1;
  while (a > 0)
    {
      int t = i / a, x = a;
      a = i % x;
      i = x;
      x = d;
      d = v - t * x;
      v = x;
    }
  v %= n;
  if (v < 0)
    v = (v + n) % n;
  return v;
}

/* src/utils.cc:243-248 */
static int o_floor_to_pow2(double x)
{
  unsigned int ans;
  for (ans = 1; ans <= x; ans <<= 1);
  return ans / 2;
}

/* src/computefourier-1.0-2.0.cc:43-46 */
static inline int o_timesmod(int x, int a, int n)
{
  return (int)((((long long)x) * a) % n);
}

/* 32-bit wrapping product, what the reference's int overflows compute
 * (src/computefourier-3.0.cc:381-382, :743, :807). */
static inline int wrap_mul(int a, int b)
{
  return (int)(int32_t)((uint32_t)a * (uint32_t)b);
}

static int cmp_double(const void *a, const void *b)
{
  double x = *(const double *)a, y = *(const double *)b;
  return (x > y) - (x < y);
}

static int cmp_int(const void *a, const void *b)
{
  int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

/* src/utils.cc:130-158 with nth_element_immutable (:107-115): cutoff is
 * the (n-num-1)-th smallest value; take every index above it in order,
 * then indices equal to it in order until num; output ascending. */
static void o_find_largest_indices(int *output, int num, const double *samples,
                                   int n, double *tmp)
{
  memcpy(tmp, samples, sizeof(double) * n);
  qsort(tmp, n, sizeof(double), cmp_double);
  double cutoff = tmp[n - num - 1];
  int count = 0;
  for (int i = 0; i < n; i++)
    if (samples[i] > cutoff)
      output[count++] = i;
  if (count < num)
    {
      for (int i = 0; i < n; i++)
        if (samples[i] == cutoff)
          {
            output[count++] = i;
            if (count >= num)
              break;
          }
      qsort(output, count, sizeof(int), cmp_int);
    }
}

/* ------------------------------------------------------ parameter tables -- */

/* Data of src/parameters.cc:24-513: per key, Bcst_loc, Bcst_est, Comb_cst,
 * comb_loops, est_loops, loc_loops, threshold_loops, tol_loc, tol_est. */
typedef struct
{
  int key;
  double bl, be, cc;
  int cl, el, ll, tl;
  double tol_l, tol_e;
} prow;

static const prow N_COMB[] = {
  {8192, 2, 2, 32, 8, 16, 7, 6, 1e-8, 1e-8},
  {16384, 4, 4, 32, 8, 10, 6, 5, 1e-8, 1e-8},
  {32768, 4, 2, 64, 4, 8, 5, 4, 1e-8, 1e-8},
  {65536, 4, 2, 128, 6, 10, 4, 2, 1e-8, 1e-8},
  {131072, 1, 1, 8, 2, 12, 4, 3, 1e-6, 1e-8},
  {262144, 1, 1, 8, 2, 14, 5, 4, 1e-6, 1e-8},
  {524288, 0.5, 0.5, 8, 1, 10, 4, 3, 1e-6, 1e-8},
  {1048576, 0.5, 0.5, 8, 2, 12, 4, 2, 1e-6, 1e-8},
  {2097152, 0.5, 0.2, 8, 1, 10, 3, 2, 1e-6, 1e-8},
  {4194304, 0.5, 0.2, 8, 1, 8, 3, 2, 1e-6, 1e-8},
  {8388608, 0.5, 0.2, 8, 1, 8, 3, 2, 1e-6, 1e-8},
  {16777216, 0.5, 0.2, 16, 1, 8, 3, 2, 1e-6, 1e-8},
};

static const prow N_PLAIN[] = {
  {8192, 2, 2, 1, 1, 16, 7, 6, 1e-8, 1e-8},
  {16384, 4, 4, 1, 1, 10, 6, 5, 1e-8, 1e-8},
  {32768, 4, 2, 1, 1, 8, 5, 4, 1e-8, 1e-8},
  {65536, 4, 2, 1, 1, 8, 5, 4, 1e-8, 1e-8},
  {131072, 2, 1, 1, 1, 10, 5, 4, 1e-6, 1e-8},
  {262144, 2, 0.5, 1, 1, 14, 4, 3, 1e-6, 1e-8},
  {524288, 1, 0.5, 1, 1, 12, 5, 4, 1e-6, 1e-8},
  {1048576, 2, 0.5, 1, 1, 12, 4, 3, 1e-6, 1e-8},
  {2097152, 2, 0.2, 1, 1, 15, 3, 2, 1e-6, 1e-8},
  {4194304, 4, 0.2, 1, 1, 10, 3, 2, 1e-6, 1e-8},
  {8388608, 2, 0.2, 1, 1, 8, 3, 2, 1e-6, 1e-8},
  {16777216, 4, 0.2, 1, 1, 8, 3, 2, 1e-6, 1e-8},
};

static const prow K_COMB[] = {
  {50, 0.5, 0.2, 16, 1, 10, 3, 2, 1e-6, 1.0e-8},
  {100, 0.5, 0.2, 16, 1, 12, 4, 2, 1e-6, 1.0e-8},
  {200, 0.5, 0.5, 32, 1, 8, 4, 3, 1e-6, 0.5e-8},
  {500, 0.5, 0.5, 64, 1, 10, 4, 3, 1e-6, 0.5e-8},
  {1000, 1, 1, 128, 3, 12, 4, 3, 1e-6, 0.5e-8},
  {2000, 1, 1, 512, 3, 16, 4, 3, 1e-7, 0.2e-8},
  {2500, 1, 1, 512, 3, 16, 4, 3, 1e-7, 0.2e-8},
  {4000, 1, 2, 512, 3, 14, 8, 7, 1e-8, 0.5e-8},
};

static const prow K_PLAIN[] = {
  {50, 4, 0.2, 1, 1, 10, 3, 2, 1e-6, 1.0e-8},
  {100, 2, 0.2, 1, 1, 12, 3, 2, 1e-6, 1.0e-8},
  {200, 4, 0.5, 1, 1, 10, 3, 2, 1e-6, 0.5e-8},
  {500, 2, 1, 1, 1, 12, 4, 3, 1e-6, 0.5e-8},
  {1000, 2, 1, 1, 1, 12, 5, 4, 1e-6, 1.0e-8},
  {2000, 2, 1, 1, 1, 16, 5, 4, 1e-7, 0.5e-8},
  {2500, 2, 1, 1, 1, 16, 5, 4, 1e-7, 0.5e-8},
  {4000, 2, 2, 1, 1, 14, 6, 5, 1e-8, 1.0e-8},
};

static const prow *lookup(const prow *t, int len, int key)
{
  for (int i = 0; i < len; i++)
    if (t[i].key == key)
      return &t[i];
  return NULL;
}

/* ---------------------------------------------------------------- filters -- */

/* src/filters.cc:62-68 */
static double o_cheb(double m, double x)
{
  if (fabs(x) <= 1)
    return cos(m * acos(x));
  else
    return creal(ccosh(m * cacosh(x)));
}

/* src/filters.cc:70-86; returns 2*w doubles. */
static double *o_make_dolphchebyshev_t(double lobefrac, double tolerance, int *w_out)
{
  int w = (int)((1 / M_PI) * (1 / lobefrac) * acosh(1. / tolerance));
  if (!(w % 2))
    w--;
  double *x = (double *)malloc(sizeof(double) * 2 * (size_t)w);
  double t0 = cosh(acosh(1 / tolerance) / (w - 1));
  for (int i = 0; i < w; i++)
    {
      x[2 * i] = o_cheb(w - 1, t0 * cos(M_PI * i / w)) * tolerance;
      x[2 * i + 1] = 0.0;
    }
  shim_fft(w, x, -1);
  /* shift(x, w, w/2) (src/utils.cc:28-37): x[i] <- x[i - r], then real part */
  int r = w / 2;
  double *y = (double *)malloc(sizeof(double) * 2 * (size_t)w);
  for (int i = 0; i < w; i++)
    {
      int src = (i - r + w) % w;
      y[2 * i] = x[2 * src];
      y[2 * i + 1] = 0.0;
    }
  free(x);
  *w_out = w;
  return y;
}

/* src/filters.cc:109-160.  x (2*w doubles) is replaced by the time taps;
 * returns the n-point freq array (2*n doubles). */
static double *o_make_multiple_t(double *x, int w, int n, int b)
{
  double *g = (double *)calloc(2 * (size_t)n, sizeof(double));
  double *h = (double *)malloc(sizeof(double) * 2 * (size_t)n);
  memcpy(g, x + 2 * (w / 2), sizeof(double) * 2 * (size_t)(w - w / 2));
  memcpy(g + 2 * (size_t)(n - w / 2), x, sizeof(double) * 2 * (size_t)(w / 2));
  shim_fft(n, g, -1);
  double sr = 0, si = 0;
  for (int i = 0; i < b; i++)
    {
      sr += g[2 * i];
      si += g[2 * i + 1];
    }
  double max = 0;
  int offset = b / 2;
  for (int i = 0; i < n; i++)
    {
      long d = ((long)i + n + offset) % n;
      h[2 * d] = sr;
      h[2 * d + 1] = si;
      double m = hypot(sr, si);         /* cabs */
      max = (max < m) ? m : max;        /* std::max(max, cabs(s)) */
      long ib = ((long)i + b) % n;
      double dr = g[2 * ib] - g[2 * i], di = g[2 * ib + 1] - g[2 * i + 1];
      sr = sr + dr;
      si = si + di;
    }
  for (long i = 0; i < n; i++)
    {
      h[2 * i] /= max;
      h[2 * i + 1] /= max;
    }
  double complex step = cexp(-2 * M_PI * I * (w / 2) / n);
  double str = creal(step), sti = cimag(step);
  double ocr = 1.0, oci = 0.0;
  for (long i = 0; i < n; i++)
    {
      double a = h[2 * i], bb = h[2 * i + 1];
      h[2 * i] = a * ocr - bb * oci;
      h[2 * i + 1] = a * oci + bb * ocr;
      double nr = ocr * str - oci * sti, ni = ocr * sti + oci * str;
      ocr = nr;
      oci = ni;
    }
  memcpy(g, h, sizeof(double) * 2 * (size_t)n);
  shim_fft(n, g, +1);
  for (int i = 0; i < w; i++)
    {
      x[2 * i] = g[2 * i] / n;
      x[2 * i + 1] = g[2 * i + 1] / n;
    }
  free(g);
  return h;
}

/* ------------------------------------------------------------------ plan -- */

typedef struct
{
  /* v1 / v2 */
  int *a, *ai;
  double *x_samp, *x_sampt, *samples;
  int *score, *hits, *J, *comb, *Jall;
  long hits_found;
  int num_comb;
  double *comb_xs, *comb_samples;
  int *pa_first, *pa_second;
  double *nth_tmp;
  /* v3 */
  double *man, *gauss, *gperm, *perm_x;
  int *est_f;
  double *est_v;
  int v3dbg[8];
  /* v3 trace: per found tone (round, stage, key, value) */
  double *trace;
  long trace_n, trace_cap;
} oscratch;

struct oracle_plan
{
  int version, n, k;
  int B_loc, B_thresh, B_est, W_Comb, Comb_loops;
  int loops_loc, loops_thresh, loops_est;
  int w_loc, w_est;
  double *t_loc, *f_loc, *t_est, *f_est;
  long x_samp_size;
  int B_g1, w_g1, B_g2, w_g2, W_Man, Gauss_loops, Gauss2_loops, Man_loops;
  int nthreads;
  oscratch *scr;
};

static int is_pow2(long x)
{
  return x > 0 && (x & (x - 1)) == 0;
}

static void alloc_scratch(oracle_plan *p, oscratch *s)
{
  int n = p->n;
  memset(s, 0, sizeof(*s));
  if (p->version < 2)
    {
      int L = p->loops_loc + p->loops_est;
      int cap = MAXI(MAXI(p->B_loc, p->B_est), p->W_Comb);
      s->a = (int *)calloc(L, sizeof(int));
      s->ai = (int *)calloc(L, sizeof(int));
      s->x_samp = (double *)calloc(2 * (size_t)p->x_samp_size, sizeof(double));
      s->x_sampt = (double *)calloc(2 * (size_t)p->x_samp_size, sizeof(double));
      s->samples = (double *)calloc((size_t)p->x_samp_size, sizeof(double));
      s->score = (int *)calloc((size_t)n, sizeof(int));
      s->hits = (int *)calloc(2 * (size_t)n, sizeof(int));
      s->J = (int *)calloc(p->B_thresh, sizeof(int));
      s->Jall = (int *)calloc((size_t)L * p->B_thresh, sizeof(int));
      s->comb = (int *)calloc((size_t)p->Comb_loops * p->B_thresh, sizeof(int));
      s->comb_xs = (double *)calloc(2 * (size_t)p->W_Comb, sizeof(double));
      s->comb_samples = (double *)calloc((size_t)p->W_Comb, sizeof(double));
      s->pa_first = (int *)calloc((size_t)p->Comb_loops * p->B_thresh, sizeof(int));
      s->pa_second = (int *)calloc((size_t)p->Comb_loops * p->B_thresh, sizeof(int));
      s->nth_tmp = (double *)calloc(cap, sizeof(double));
    }
  else
    {
      int cap = MAXI(MAXI(p->W_Man, p->B_g1), p->B_g2);
      s->man = (double *)calloc(4 * (size_t)p->W_Man, sizeof(double));
      s->gauss = (double *)calloc(4 * (size_t)p->B_g1, sizeof(double));
      s->gperm = (double *)calloc(4 * (size_t)p->B_g2, sizeof(double));
      s->perm_x = (double *)calloc(2 * (size_t)(p->w_g2 + 1), sizeof(double));
      s->est_f = (int *)calloc(cap, sizeof(int));
      s->est_v = (double *)calloc(2 * (size_t)cap, sizeof(double));
      s->trace_cap = 1 << 16;
      s->trace = (double *)calloc(5 * (size_t)s->trace_cap, sizeof(double));
    }
}

static void trace_add(oscratch *s, int round, int stage, int key, double re, double im)
{
  if (s->trace_n < s->trace_cap)
    {
      double *t = s->trace + 5 * s->trace_n;
      t[0] = round;
      t[1] = stage;
      t[2] = key;
      t[3] = re;
      t[4] = im;
    }
  s->trace_n++;
}

static void free_scratch(oscratch *s)
{
  void *ptrs[] = { s->a, s->ai, s->x_samp, s->x_sampt, s->samples, s->score,
    s->hits, s->J, s->Jall, s->comb, s->comb_xs, s->comb_samples,
    s->pa_first, s->pa_second, s->nth_tmp, s->man, s->gauss, s->gperm,
    s->perm_x, s->est_f, s->est_v, s->trace
  };
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++)
    free(ptrs[i]);
}

/* src/sfft.cc:298-420 */
static int make_plan_v1v2(oracle_plan *p, unsigned n, unsigned k, int with_comb)
{
  double Bcst_loc = 1, Bcst_est = 1, Comb_cst = 2;
  int loc_loops = 4, est_loops = 16, threshold_loops = 3, comb_loops = 1;
  double tolerance_loc = 1.e-8, tolerance_est = 1.e-8;
  const prow *r;
  if (k > 50)
    r = with_comb ? lookup(K_COMB, 8, (int)n) : lookup(K_PLAIN, 8, (int)n);
  else
    r = with_comb ? lookup(N_COMB, 12, (int)n) : lookup(N_PLAIN, 12, (int)n);
  if (r)
    {
      Bcst_loc = r->bl;
      Bcst_est = r->be;
      Comb_cst = r->cc;
      comb_loops = r->cl;
      est_loops = r->el;
      loc_loops = r->ll;
      threshold_loops = r->tl;
      tolerance_loc = r->tol_l;
      tolerance_est = r->tol_e;
    }
  n = o_floor_to_pow2(n);
  p->n = (int)n;
  double BB_loc = (unsigned)(Bcst_loc * sqrt((double)(int)n * k / (log2(n))));
  double BB_est = (unsigned)(Bcst_est * sqrt((double)(int)n * k / (log2(n))));
  double lobefrac_loc = 0.5 / (BB_loc);
  double lobefrac_est = 0.5 / (BB_est);
  int b_loc = (int)(1.2 * 1.1 * ((double)n / BB_loc));
  int b_est = (int)(1.4 * 1.1 * ((double)n / BB_est));
  p->B_loc = o_floor_to_pow2(BB_loc);
  p->B_thresh = 2 * k;
  p->B_est = o_floor_to_pow2(BB_est);
  p->W_Comb = o_floor_to_pow2(Comb_cst * n / p->B_loc);
  p->Comb_loops = comb_loops;
  p->loops_loc = loc_loops;
  p->loops_thresh = threshold_loops;
  p->loops_est = est_loops;
  /* domain of the reference (src/utils.cc:134 asserts n >= num + 1) */
  if (p->B_loc < p->B_thresh + 1 || p->B_est < p->B_thresh + 1)
    return -1;
  if (with_comb && p->W_Comb < p->B_thresh + 1)
    return -1;
  if (p->W_Comb < 1 || (int)n % p->W_Comb)
    return -1;
  p->t_loc = o_make_dolphchebyshev_t(lobefrac_loc, tolerance_loc, &p->w_loc);
  p->t_est = o_make_dolphchebyshev_t(lobefrac_est, tolerance_est, &p->w_est);
  if (p->w_loc > (int)n || p->w_est > (int)n || b_loc > (int)n || b_est > (int)n)
    return -1;
  p->f_loc = o_make_multiple_t(p->t_loc, p->w_loc, n, b_loc);
  p->f_est = o_make_multiple_t(p->t_est, p->w_est, n, b_est);
  p->x_samp_size = (long)p->loops_loc * p->B_loc + (long)p->loops_est * p->B_est;
  return 0;
}

/* src/sfft.cc:506-579 */
static int make_plan_v3(oracle_plan *p, unsigned n, unsigned k)
{
  double Bcst = 1, Bcst2 = 0.25, Mancst = 10;
  p->Gauss_loops = 2;
  p->Gauss2_loops = 2;
  p->Man_loops = 2;
  double tolerance_g1 = 1.e-8, tolerance_g2 = 1.e-8;
  n = o_floor_to_pow2(n);
  p->n = (int)n;
  p->W_Man = o_floor_to_pow2(Mancst * ((double)k));
  p->W_Man = MINI(n / 2, (unsigned)p->W_Man);
  double BB = (unsigned)(Bcst * ((double)k));
  p->B_g1 = o_floor_to_pow2(BB);
  double lobefrac_g1 = 0.5 / (BB);
  int b_g1 = (int)(1.00 * ((double)n / p->B_g1));
  double BB2 = (unsigned)(Bcst2 * ((double)k));
  p->B_g2 = o_floor_to_pow2(BB2);
  /* k < 8 gives B_g2 < 2: outside the reference's working range */
  if (p->B_g2 < 2 || p->W_Man < 2)
    return -1;
  double lobefrac_g2 = 0.5 / (BB2);
  int b_g2 = (int)(1.00 * ((double)n / p->B_g2));
  p->t_loc = o_make_dolphchebyshev_t(lobefrac_g1, tolerance_g1, &p->w_g1);
  p->t_est = o_make_dolphchebyshev_t(lobefrac_g2, tolerance_g2, &p->w_g2);
  if (p->w_g1 > (int)n || p->w_g2 + 2 > (int)n)
    return -1;
  p->f_loc = o_make_multiple_t(p->t_loc, p->w_g1, n, b_g1);
  p->f_est = o_make_multiple_t(p->t_est, p->w_g2, n, b_g2);
  return 0;
}

oracle_plan *oracle_make_plan(int n, int k, int version)
{
  if (n < 16 || !is_pow2(n) || k < 1 || version < 0 || version > 2)
    return NULL;
  oracle_plan *p = (oracle_plan *)calloc(1, sizeof(*p));
  p->version = version;
  p->k = k;
  int rc = (version < 2) ? make_plan_v1v2(p, n, k, version == 1)
    : make_plan_v3(p, n, k);
  if (rc)
    {
      free(p->t_loc);
      free(p->t_est);
      free(p->f_loc);
      free(p->f_est);
      free(p);
      return NULL;
    }
#ifdef _OPENMP
  p->nthreads = omp_get_max_threads();
#else
  p->nthreads = 1;
#endif
  p->scr = (oscratch *)calloc(p->nthreads, sizeof(oscratch));
  for (int i = 0; i < p->nthreads; i++)
    alloc_scratch(p, &p->scr[i]);
  return p;
}

void oracle_get_params(const oracle_plan *p, oracle_params *o)
{
  memset(o, 0, sizeof(*o));
  o->version = p->version;
  o->n = p->n;
  o->k = p->k;
  o->B_loc = p->B_loc;
  o->B_thresh = p->B_thresh;
  o->B_est = p->B_est;
  o->W_Comb = p->W_Comb;
  o->Comb_loops = p->Comb_loops;
  o->loops_loc = p->loops_loc;
  o->loops_thresh = p->loops_thresh;
  o->loops_est = p->loops_est;
  o->w_loc = p->w_loc;
  o->w_est = p->w_est;
  o->x_samp_size = p->x_samp_size;
  o->B_g1 = p->B_g1;
  o->w_g1 = p->w_g1;
  o->B_g2 = p->B_g2;
  o->w_g2 = p->w_g2;
  o->W_Man = p->W_Man;
  o->Gauss_loops = p->Gauss_loops;
  o->Gauss2_loops = p->Gauss2_loops;
  o->Man_loops = p->Man_loops;
}

const double *oracle_filter_time(const oracle_plan *p, int which)
{
  return which ? p->t_est : p->t_loc;
}

const double *oracle_filter_freq(const oracle_plan *p, int which)
{
  return which ? p->f_est : p->f_loc;
}

void oracle_free_plan(oracle_plan *p)
{
  if (!p)
    return;
  for (int i = 0; i < p->nthreads; i++)
    free_scratch(&p->scr[i]);
  free(p->scr);
  free(p->t_loc);
  free(p->t_est);
  free(p->f_loc);
  free(p->f_est);
  free(p);
}

/* ----------------------------------------------------------------- v1/v2 -- */

/* src/computefourier-1.0-2.0.cc:48-82 */
static void o_comb_filt(oracle_plan *p, oscratch *s, const double *x, int *approved)
{
  int n = p->n, W = p->W_Comb, num = p->B_thresh;
  int sigma = n / W;
  int offset = (unsigned)floor(drand48() * sigma);
  for (int i = 0; i < W; i++)
    {
      s->comb_xs[2 * i] = x[2 * ((long)offset + (long)i * sigma)];
      s->comb_xs[2 * i + 1] = x[2 * ((long)offset + (long)i * sigma) + 1];
    }
  shim_fft(W, s->comb_xs, -1);
  for (int i = 0; i < W; i++)
    {
      double re = s->comb_xs[2 * i], im = s->comb_xs[2 * i + 1];
      s->comb_samples[i] = re * re + im * im;
    }
  o_find_largest_indices(approved, num, s->comb_samples, W, s->nth_tmp);
}

static void add_hit(oscratch *s, int loc, int thresh)
{
  s->score[loc]++;
  if (s->score[loc] == thresh)
    s->hits[s->hits_found++] = loc;
}

/* src/computefourier-1.0-2.0.cc:91-116 */
static void o_filter_regular(oracle_plan *p, oscratch *s, const int *J, int B, int a)
{
  int n = p->n, num = p->B_thresh;
  for (int i = 0; i < num; i++)
    {
      int low = ((int)(ceil((J[i] - 0.5) * n / B)) + n) % n;
      int high = ((int)(ceil((J[i] + 0.5) * n / B)) + n) % n;
      int loc = o_timesmod(low, a, n);
      for (int j = low; j != high; j = (j + 1) % n)
        {
          add_hit(s, loc, p->loops_thresh);
          loc = (loc + a) % n;
        }
    }
}

static int cmp_pair(const void *x, const void *y)
{
  const int *a = (const int *)x, *b = (const int *)y;
  if (a[0] != b[0])
    return (a[0] > b[0]) - (a[0] < b[0]);
  return (a[1] > b[1]) - (a[1] < b[1]);
}

/* src/computefourier-1.0-2.0.cc:125-184 */
static void o_filter_comb(oracle_plan *p, oscratch *s, const int *J, int B, int a, int ai)
{
  int n = p->n, num = p->B_thresh, W = p->W_Comb, nc = s->num_comb;
  int *pairs = (int *)malloc(sizeof(int) * 2 * (size_t)nc);
  for (int m = 0; m < nc; m++)
    {
      int prev = o_timesmod(s->comb[m], ai, W);
      pairs[2 * m] = prev;
      pairs[2 * m + 1] = o_timesmod(prev, a, n);
    }
  qsort(pairs, nc, 2 * sizeof(int), cmp_pair);
  for (int i = 0; i < num; i++)
    {
      int low = ((int)(ceil((J[i] - 0.5) * n / B)) + n) % n;
      int high = ((int)(ceil((J[i] + 0.5) * n / B)) + n) % n;
      /* upper_bound of (low % W, -1) in the sorted pairs */
      int key = low % W, index = 0;
      while (index < nc && pairs[2 * index] < key)
        index++;
      int location = low - (low % W);
      int locinv = o_timesmod(location, a, n);
      for (int j = index;; j++)
        {
          if (j == nc)
            {
              j -= nc;
              location = (location + W) % n;
              locinv = o_timesmod(location, a, n);
            }
          int approved_loc = location + pairs[2 * j];
          if ((low < high && (approved_loc >= high || approved_loc < low)) ||
              (low > high && (approved_loc >= high && approved_loc < low)))
            break;
          int loc = (locinv + pairs[2 * j + 1]) % n;
          add_hit(s, loc, p->loops_thresh);
        }
    }
  free(pairs);
}

/* src/computefourier-1.0-2.0.cc:195-327 */
static void o_inner_loop_locate(oracle_plan *p, oscratch *s, const double *x)
{
  int n = p->n, L = p->loops_loc + p->loops_est, Lloc = p->loops_loc;
  memset(s->x_sampt, 0, sizeof(double) * 2 * (size_t)p->x_samp_size);
  for (int j = 0; j < L; j++)
    {
      int loc = (j < Lloc);
      const double *ft = loc ? p->t_loc : p->t_est;
      int w = loc ? p->w_loc : p->w_est;
      int B = loc ? p->B_loc : p->B_est;
      long off = (long)MINI(j, Lloc) * p->B_loc + (long)MAXI(0, j - Lloc) * p->B_est;
      double *xs = s->x_sampt + 2 * off;
      long index = 0;           /* b = 0 */
      for (int t = 0; t < w; t++)
        {
          double a = x[2 * index], b = x[2 * index + 1];
          double c = ft[2 * t], d = ft[2 * t + 1];
          double re = a * c - b * d;
          double im = a * d + b * c;
          int bk = t & (B - 1);
          xs[2 * bk] = xs[2 * bk] + re;
          xs[2 * bk + 1] = xs[2 * bk + 1] + im;
          index = (index + s->ai[j]) & (n - 1);
        }
    }
  /* batched forward FFTs, out of place into x_samp (src/sfft.cc:274-295) */
  memcpy(s->x_samp, s->x_sampt, sizeof(double) * 2 * (size_t)p->x_samp_size);
  for (int j = 0; j < L; j++)
    {
      int loc = (j < Lloc);
      int B = loc ? p->B_loc : p->B_est;
      long off = (long)MINI(j, Lloc) * p->B_loc + (long)MAXI(0, j - Lloc) * p->B_est;
      shim_fft(B, s->x_samp + 2 * off, -1);
    }
  for (long j = 0; j < p->x_samp_size; j++)
    {
      double re = s->x_samp[2 * j], im = s->x_samp[2 * j + 1];
      s->samples[j] = re * re + im * im;
    }
  for (int j = 0; j < L; j++)
    {
      int loc = (j < Lloc);
      int B = loc ? p->B_loc : p->B_est;
      long off = (long)MINI(j, Lloc) * p->B_loc + (long)MAXI(0, j - Lloc) * p->B_est;
      o_find_largest_indices(s->J, p->B_thresh, s->samples + off, B, s->nth_tmp);
      memcpy(s->Jall + (size_t)j * p->B_thresh, s->J, sizeof(int) * p->B_thresh);
      if (loc)
        {
          if (p->version == 0)
            o_filter_regular(p, s, s->J, B, s->a[j]);
          else
            o_filter_comb(p, s, s->J, B, s->a[j], s->ai[j]);
        }
    }
}

/* src/computefourier-1.0-2.0.cc:340-419; writes (re, im) per hit into vals. */
static void o_estimate_values(oracle_plan *p, oscratch *s, double *vals)
{
  int n = p->n, L = p->loops_loc + p->loops_est, Lloc = p->loops_loc;
  double re[64], im[64];
  for (long i = 0; i < s->hits_found; i++)
    {
      int f = s->hits[i];
      for (int j = 0; j < L; j++)
        {
          long off = (long)MINI(j, Lloc) * p->B_loc + (long)MAXI(0, j - Lloc) * p->B_est;
          int B = (j < Lloc) ? p->B_loc : p->B_est;
          const double *freq = (j < Lloc) ? p->f_loc : p->f_est;
          int permuted_index = o_timesmod(s->ai[j], f, n);
          int hashed_to = permuted_index / (n / B);
          int dist = permuted_index % (n / B);
          if (dist > (n / B) / 2)
            {
              hashed_to = (hashed_to + 1) % B;
              dist -= n / B;
            }
          dist = (n - dist) % n;
          double a = s->x_samp[2 * (off + hashed_to)];
          double b = s->x_samp[2 * (off + hashed_to) + 1];
          double c = freq[2 * (long)dist], d = freq[2 * (long)dist + 1];
          double den = c * c + d * d;
          re[j] = (a * c + b * d) / den;
          im[j] = (a * d - b * c) / den;        /* the reference's sign: conj */
        }
      int location = (L - 1) / 2;
      qsort(re, L, sizeof(double), cmp_double);
      qsort(im, L, sizeof(double), cmp_double);
      vals[2 * i] = re[location];
      vals[2 * i + 1] = im[location];
    }
}

/* src/computefourier-1.0-2.0.cc:437-541 */
static void o_outer_loop(oracle_plan *p, oscratch *s, const double *x, double **vals_out)
{
  int n = p->n, L = p->loops_loc + p->loops_est, num = p->B_thresh;
  memset(s->score, 0, sizeof(int) * (size_t)n);
  for (int i = 0; i < L; i++)
    {
      int a = 0;
      while (o_gcd(a, n) != 1)
        a = (int)(random() % n);
      s->a[i] = a;
      s->ai[i] = o_mod_inverse(a, n);
    }
  s->hits_found = 0;
  s->num_comb = num;
  if (p->version == 1)
    {
      for (int i = 0; i < p->Comb_loops; i++)
        o_comb_filt(p, s, x, s->comb + (size_t)i * num);
      if (p->Comb_loops > 1)
        {
          int tot = p->Comb_loops * num;
          qsort(s->comb, tot, sizeof(int), cmp_int);
          int last = 0;
          for (int i = 1; i < tot; i++)
            if (s->comb[i] != s->comb[last])
              s->comb[++last] = s->comb[i];
          s->num_comb = last + 1;
        }
      long nw = n / p->W_Comb;
      s->hits_found = (long)s->num_comb * nw;
      for (long j = 0; j < nw; j++)
        for (int i = 0; i < s->num_comb; i++)
          s->hits[j * s->num_comb + i] = (int)(j * p->W_Comb + s->comb[i]);
    }
  o_inner_loop_locate(p, s, x);
  double *vals = (double *)malloc(sizeof(double) * 2 * (size_t)(s->hits_found + 1));
  o_estimate_values(p, s, vals);
  *vals_out = vals;
}

/* -------------------------------------------------------------------- v3 -- */

typedef struct
{
  int *keys;
  double *vals;
  long count, cap;
  long *table;                  /* open addressing: index+1, 0 = empty */
  long tcap;
} omap;

static void omap_init(omap *m)
{
  m->cap = 1024;
  m->count = 0;
  m->keys = (int *)malloc(sizeof(int) * m->cap);
  m->vals = (double *)malloc(sizeof(double) * 2 * m->cap);
  m->tcap = 4096;
  m->table = (long *)calloc(m->tcap, sizeof(long));
}

static void omap_free(omap *m)
{
  free(m->keys);
  free(m->vals);
  free(m->table);
}

static long omap_slot(const omap *m, int key)
{
  unsigned long h = ((unsigned long)(unsigned)key * 2654435761UL) & (m->tcap - 1);
  while (m->table[h] && m->keys[m->table[h] - 1] != key)
    h = (h + 1) & (m->tcap - 1);
  return (long)h;
}

/* operator[] of the reference's map: insert (0, 0) when absent. */
static long omap_get(omap *m, int key)
{
  long h = omap_slot(m, key);
  if (m->table[h])
    return m->table[h] - 1;
  if (m->count == m->cap)
    {
      m->cap *= 2;
      m->keys = (int *)realloc(m->keys, sizeof(int) * m->cap);
      m->vals = (double *)realloc(m->vals, sizeof(double) * 2 * m->cap);
    }
  if (2 * (m->count + 1) > m->tcap)
    {
      free(m->table);
      m->tcap *= 2;
      m->table = (long *)calloc(m->tcap, sizeof(long));
      for (long i = 0; i < m->count; i++)
        m->table[omap_slot(m, m->keys[i])] = i + 1;
      h = omap_slot(m, key);
    }
  long idx = m->count++;
  m->keys[idx] = key;
  m->vals[2 * idx] = 0.0;
  m->vals[2 * idx + 1] = 0.0;
  m->table[h] = idx + 1;
  return idx;
}

/* src/computefourier-3.0.cc:66-87 */
static void o_permute_fourier(double *dest, int w, const double *src, int n,
                              int offset, int ai, int b)
{
  double complex shift = cos(2 * M_PI * offset * b / n) + I * sin(2 * M_PI * offset * b / n);
  double complex step = cos(2 * M_PI * ai * b / n) + I * sin(2 * M_PI * ai * b / n);
  int index = offset % n;
  for (int i = 0; i < w; i++)
    {
      double complex v = CMPLX(src[2 * index], src[2 * index + 1]);
      double complex r = v * shift;
      dest[2 * i] = creal(r);
      dest[2 * i + 1] = cimag(r);
      shift = shift * step;
      index = (index + ai) % n;
    }
}

/* src/computefourier-3.0.cc:96-127 */
static void o_mansour_filt(oracle_plan *p, oscratch *s, const double *x, int init_offset)
{
  int n = p->n, W = p->W_Man, n1 = n - 1, sigma = n / W;
  int index = init_offset, index_p1 = (init_offset + 1) & n1;
  for (int i = 0; i < W; i++)
    {
      s->man[4 * i] = x[2 * index];
      s->man[4 * i + 1] = x[2 * index + 1];
      s->man[4 * i + 2] = x[2 * index_p1];
      s->man[4 * i + 3] = x[2 * index_p1 + 1];
      index = (index + sigma) & n1;
      index_p1 = (index_p1 + sigma) & n1;
    }
  int sz[2] = { W, W };
  fftw_plan pl = fftw_plan_many_dft(1, sz, 2, (fftw_complex *)s->man, NULL, 2, 1,
                                    (fftw_complex *)s->man, NULL, 2, 1, FFTW_FORWARD, FFTW_ESTIMATE);
  fftw_execute(pl);
  fftw_destroy_plan(pl);
}

/* Two-shift fold shared by src/computefourier-3.0.cc:130-212 and :215-297:
 * bucket (t mod B) of shift l accumulates s_l(t) * filter[t] over the
 * floor(w/B) full chunks only (A.11). */
static void o_gauss_fold(const double *src0, const double *src1, long stride_mask,
                         long base, int use_index, const double *filter, int w,
                         int B, double *G)
{
  memset(G, 0, sizeof(double) * 4 * (size_t)B);
  unsigned chunks = (unsigned)(2 * w) / (unsigned)(2 * B);
  for (unsigned chunk = 0; chunk < chunks; chunk++)
    {
      long start = (long)chunk * B;
      long end = MINI((long)(chunk + 1) * B, (long)w);
      for (long t = start; t < end; t++)
        {
          long i0, i1;
          if (use_index)
            {
              i0 = (base + t) & stride_mask;
              i1 = (base + 1 + t) & stride_mask;
            }
          else
            {
              i0 = t;
              i1 = t + 1;
            }
          double a0 = src0[2 * i0], b0 = src0[2 * i0 + 1];
          double a1 = src1[2 * i1], b1 = src1[2 * i1 + 1];
          double c = filter[2 * t], d = filter[2 * t + 1];
          double ac0 = c * a0, ad0 = d * a0, bc0 = c * b0, bd0 = d * b0;
          double ac1 = c * a1, ad1 = d * a1, bc1 = c * b1, bd1 = d * b1;
          long bk = t - start;
          G[4 * bk] = G[4 * bk] + (ac0 - bd0);
          G[4 * bk + 1] = G[4 * bk + 1] + (ad0 + bc0);
          G[4 * bk + 2] = G[4 * bk + 2] + (ac1 - bd1);
          G[4 * bk + 3] = G[4 * bk + 3] + (ad1 + bc1);
        }
    }
  int sz[2] = { B, B };
  fftw_plan pl = fftw_plan_many_dft(1, sz, 2, (fftw_complex *)G, NULL, 2, 1,
                                    (fftw_complex *)G, NULL, 2, 1, FFTW_FORWARD, FFTW_ESTIMATE);
  fftw_execute(pl);
  fftw_destroy_plan(pl);
}

/* src/computefourier-3.0.cc:300-351 */
static void o_update_mansour(int key, double vr, double vi, double *SAMP, int n,
                             int W, int offset)
{
  const double PI2_OVER_N = 2 * M_PI / n;
  int h = key & (W - 1);
  double arg0 = PI2_OVER_N * key * offset, arg1 = PI2_OVER_N * key * (offset + 1);
  double cpi[2] = { sin(arg0), sin(arg1) }, cpr[2] = { cos(arg0), cos(arg1) };
  for (int l = 0; l < 2; l++)
    {
      double a0 = vr * cpr[l], b0 = vi * cpi[l], c0 = a0 - b0;
      double rr = (double)W * c0;
      double a1 = vr * cpi[l], b1 = vi * cpr[l], c1 = a1 + b1;
      double ri = (double)W * c1;
      SAMP[4 * h + 2 * l] = SAMP[4 * h + 2 * l] - rr;
      SAMP[4 * h + 2 * l + 1] = SAMP[4 * h + 2 * l + 1] - ri;
    }
}

/* src/computefourier-3.0.cc:354-463 */
static void o_update_gaussian(int key, double a1, double b1, double *SAMP,
                              const double *filterf, int n, int B, int init_G_offset,
                              int step)
{
  const double PI2_DIV_N = 2 * M_PI / n;
  const int n1 = n - 1;
  unsigned n_over_B = n / B;
  int hashed_to = (int)(key * 1. / n_over_B + 0.5) % B;
  int dist1 = (int)(((unsigned)hashed_to * n_over_B - (unsigned)key + (unsigned)n) & (unsigned)n1);
  int dist2 = (int)(((unsigned)dist1 + (unsigned)n + n_over_B) & (unsigned)n1);
  int dist3 = (int)(((unsigned)dist1 + (unsigned)n + (unsigned)n - n_over_B) & (unsigned)n1);
  int key_offset = wrap_mul(key, init_G_offset) % n;
  int key_offset2 = wrap_mul(key, (int)((uint32_t)init_G_offset + (uint32_t)step)) % n;
  double arg0 = PI2_DIV_N * key_offset, arg1 = PI2_DIV_N * key_offset2;
  double a2 = cos(arg0), b2 = sin(arg0), a22 = cos(arg1), b22 = sin(arg1);
  double v1r = a1 * a2 - b1 * b2, v1i = a1 * b2 + b1 * a2;
  double v2r = a1 * a22 - b1 * b22, v2i = a1 * b22 + b1 * a22;
  int dists[3] = { dist1, dist2, dist3 };
  int bks[3] = { hashed_to, (hashed_to + 1) % B, (hashed_to + B - 1) % B };
  double vr[2] = { v1r, v2r }, vi[2] = { v1i, v2i };
  for (int l = 0; l < 2; l++)
    for (int q = 0; q < 3; q++)
      {
        double fr = filterf[2 * (long)dists[q]], fi = filterf[2 * (long)dists[q] + 1];
        double rr = vr[l] * fr - vi[l] * fi;
        double ri = vr[l] * fi + vi[l] * fr;
        SAMP[4 * bks[q] + 2 * l] = SAMP[4 * bks[q] + 2 * l] - rr;
        SAMP[4 * bks[q] + 2 * l + 1] = SAMP[4 * bks[q] + 2 * l + 1] - ri;
      }
}

/* src/computefourier-3.0.cc:484-640 */
static int o_estimate_freq_gauss(int BUCKETS, const double *SAMP, int init_offset,
                                 int n, int a, int b, int jump, const double *filterf,
                                 int *EST_FREQS, double *EST_VALUES)
{
  const unsigned n1 = n - 1, B1 = BUCKETS - 1;
  const double PI2 = 2 * M_PI;
  const double N_OVER_PI2 = n / PI2;
  const double PI2_A_OFFSET_OVER_N = PI2 * a * init_offset / n;
  const double BUCKETS_OVER_N = (double)BUCKETS / n;
  const int N_OVER_BUCKETS = n / BUCKETS;
  const double collision_threshold = 1e-12;
  double separation = 1. / jump;
  int found = 0;
  for (int i = 0; i < BUCKETS; i += 2)
    for (int j = 0; j < 2; j++)
      {
        int bk = i + j;
        double a0 = SAMP[4 * bk], b0 = SAMP[4 * bk + 1];
        double a1 = SAMP[4 * bk + 2], b1 = SAMP[4 * bk + 3];
        double zbc = (a0 * a0 + b0 * b0) + (a1 * a1 + b1 * b1);
        if (!(zbc > 1e-8))
          continue;
        double c0 = (a0 * a0 + b0 * b0);
        double c1 = (a1 * a1 + b1 * b1);
        double d0 = atan2(b0, a0), d1 = atan2(b1, a1);
        double error_b = c1 / c0 - 1;
        double error = error_b * error_b;
        error /= n;
        if ((error < collision_threshold) && (c0 > 0.01))
          {
            double slope = (d1 - d0) * separation;
            int freq = (int)lrint(N_OVER_PI2 * slope) + n;
            freq = freq & n1;
            unsigned hashed_to = (unsigned)lrint(freq * BUCKETS_OVER_N) & B1;
            if (hashed_to == (unsigned)bk)
              {
                double median_phase = d0 - PI2_A_OFFSET_OVER_N * freq;
                c0 = sqrt(c0);
                double complex mv = CMPLX(cos(median_phase), sin(median_phase));
                mv = CMPLX(c0 * creal(mv), c0 * cimag(mv));
                int dist = (int)((hashed_to * (unsigned)N_OVER_BUCKETS - (unsigned)freq + (unsigned)n) & n1);
                double complex fv = CMPLX(filterf[2 * (long)dist], filterf[2 * (long)dist + 1]);
                mv = mv / fv;
                freq = (int)(((unsigned)(o_timesmod(freq, a, n) - b + n)) & n1);
                EST_FREQS[found] = freq;
                EST_VALUES[2 * found] = creal(mv);
                EST_VALUES[2 * found + 1] = cimag(mv);
                found++;
              }
          }
      }
  return found;
}

/* src/computefourier-3.0.cc:642-776 */
static int o_estimate_freq_mansour(int BUCKETS, const double *SAMP, int init_offset,
                                   int n, int *EST_FREQS, double *EST_VALUES)
{
  const double PI2 = 2 * M_PI;
  const double N_OVER_PI2 = n / PI2;
  const double PI2_OVER_N = PI2 / n;
  const unsigned W_Man = BUCKETS;
  const unsigned FREQ_MASK = ((n - 1) & ~(W_Man - 1));
  double NORM = 1. / BUCKETS;
  double NORM2 = NORM * NORM;
  int found = 0;
  for (int i = 0; i < BUCKETS; i += 2)
    for (int j = 0; j < 2; j++)
      {
        int bk = i + j;
        double a0 = SAMP[4 * bk], b0 = SAMP[4 * bk + 1];
        double a1 = SAMP[4 * bk + 2], b1 = SAMP[4 * bk + 3];
        double zbc = (a0 * a0 + b0 * b0) * NORM2 + (a1 * a1 + b1 * b1) * NORM2;
        if (!(zbc > 1e-8))
          continue;
        double c0 = (a0 * a0 + b0 * b0) * NORM2;
        double c1 = (a1 * a1 + b1 * b1) * NORM2;
        double d0 = atan2(b0 * NORM, a0 * NORM), d1 = atan2(b1 * NORM, a1 * NORM);
        double collision_threshold = 1e-10;
        double median_abs = c0;
        double median_abs_inv = 1. / median_abs;
        double bb = (c1 * median_abs_inv) - 1;
        double error = bb * bb;
        if ((error < n * collision_threshold) && (median_abs > 0.01))
          {
            double slope = d1 - d0;
            int freq1 = (int)lrint(slope * N_OVER_PI2);
            int freq2 = (int)((unsigned)freq1 & FREQ_MASK);
            int freq3 = freq2 | bk;
            int freq_offset = wrap_mul(freq3, init_offset);
            double median_phase = d0 - PI2_OVER_N * freq_offset;
            median_abs = sqrt(median_abs);
            double s_ = sin(median_phase), c_ = cos(median_phase);
            EST_FREQS[found] = freq3;
            EST_VALUES[2 * found] = median_abs * c_;
            EST_VALUES[2 * found + 1] = median_abs * s_;
            found++;
          }
      }
  return found;
}

/* src/computefourier-3.0.cc:784-1088.  Returns the map (empty on the
 * reference's early return, :859-860). */
static void o_alternate_fft(oracle_plan *p, oscratch *s, const double *x, omap *ans)
{
  int n = p->n, k = p->k, W = p->W_Man, B1 = p->B_g1, B2 = p->B_g2;
  double *MAN = s->man, *G1 = s->gauss, *G2 = s->gperm;
  int a = 0;
  while (o_gcd(a, n) != 1)
    a = (int)(random() % n);
  int ai = o_mod_inverse(a, n);
  int b = (int)(random() % n);
  int shift = ((wrap_mul(ai, b) % n) + n) % n;
  int init_offset = (unsigned)floor(drand48() * n);
  int init_G_offset = (unsigned)floor(drand48() * n);
  int aG = wrap_mul(a, init_G_offset);
  int jump = 1;
  int *EF = s->est_f;
  double *EV = s->est_v;
  int *dbg = s->v3dbg;
  dbg[0] = a;
  dbg[1] = ai;
  dbg[2] = b;
  dbg[3] = init_offset;
  dbg[4] = init_G_offset;
  dbg[5] = 0;
  dbg[6] = 0;

  o_mansour_filt(p, s, x, init_offset);
  s->trace_n = 0;
  int found = 0;
  int found_now = o_estimate_freq_mansour(W, MAN, init_offset, n, EF, EV);
  for (int i = 0; i < found_now; i++)
    {
      trace_add(s, -2, 0, EF[i], EV[2 * i], EV[2 * i + 1]);
      long q = omap_get(ans, EF[i]);
      ans->vals[2 * q] = EV[2 * i];
      ans->vals[2 * q + 1] = EV[2 * i + 1];
      found++;
      for (int j = 0; j < 2; j++)
        {
          MAN[2 * (j + 2 * (EF[i] % W))] = 0;
          MAN[2 * (j + 2 * (EF[i] % W)) + 1] = 0;
        }
    }
  if (found == k)
    {
      dbg[6] = 1;
      dbg[7] = found;
      ans->count = 0;           /* nothing reaches out[] */
      return;
    }

  o_gauss_fold(x, x, n - 1, init_G_offset, 1, p->t_loc, p->w_g1, B1, G1);
  for (long q = 0; q < ans->count; q++)
    o_update_gaussian(ans->keys[q], ans->vals[2 * q], ans->vals[2 * q + 1], G1,
                      p->f_loc, n, B1, init_G_offset, 1);
  found_now = o_estimate_freq_gauss(B1, G1, init_G_offset, n, 1, 0, jump, p->f_loc, EF, EV);
  for (int i = 0; i < found_now; i++)
    {
      trace_add(s, -1, 1, EF[i], EV[2 * i], EV[2 * i + 1]);
      long q = omap_get(ans, EF[i]);
      double vr = ans->vals[2 * q], vi = ans->vals[2 * q + 1];
      if (vr * vr + vi * vi == 0)
        found++;
      ans->vals[2 * q] = vr + EV[2 * i];
      ans->vals[2 * q + 1] = vi + EV[2 * i + 1];
      o_update_gaussian(EF[i], EV[2 * i], EV[2 * i + 1], G1, p->f_loc, n, B1, init_G_offset, 1);
      o_update_mansour(EF[i], EV[2 * i], EV[2 * i + 1], MAN, n, W, init_offset);
    }

  o_permute_fourier(s->perm_x, p->w_g2 + jump, x, n, init_G_offset, ai, b);
  o_gauss_fold(s->perm_x, s->perm_x, 0, 0, 0, p->t_est, p->w_g2, B2, G2);
  for (long q = 0; q < ans->count; q++)
    o_update_gaussian((o_timesmod(ans->keys[q], ai, n) + shift) % n, ans->vals[2 * q],
                      ans->vals[2 * q + 1], G2, p->f_est, n, B2, aG, jump);

  int nana = 0;
  int prev_man = 0, prev_g1 = 0, prev_g2 = 0;
  int stage = 2;                /* first pass: the second Gaussian filter */
  for (;;)
    {
      if (stage == 0)
        found_now = o_estimate_freq_mansour(W, MAN, init_offset, n, EF, EV);
      else if (stage == 1)
        found_now = o_estimate_freq_gauss(B1, G1, init_G_offset, n, 1, 0, jump, p->f_loc, EF, EV);
      else
        found_now = o_estimate_freq_gauss(B2, G2, init_G_offset, n, a, b, jump, p->f_est, EF, EV);
      for (int i = 0; i < found_now; i++)
        {
          trace_add(s, nana, stage, EF[i], EV[2 * i], EV[2 * i + 1]);
          long q = omap_get(ans, EF[i]);
          double vr = ans->vals[2 * q], vi = ans->vals[2 * q + 1];
          if (vr * vr + vi * vi == 0)
            found++;
          ans->vals[2 * q] = vr + EV[2 * i];
          ans->vals[2 * q + 1] = vi + EV[2 * i + 1];
          double er = EV[2 * i], ei = EV[2 * i + 1];
          /* UPDATE_ALL, src/computefourier-3.0.cc:465-482 */
          o_update_gaussian((o_timesmod(EF[i], ai, n) + shift) % n, er, ei, G2, p->f_est, n,
                            B2, aG, jump);
          o_update_gaussian(EF[i], er, ei, G1, p->f_loc, n, B1, init_G_offset, 1);
          o_update_mansour(EF[i], er, ei, MAN, n, W, init_offset);
        }
      /* the fixpoint test of :1040-1073 follows every Gaussian-2 pass of the
       * round-robin loop; this loop's pass 0 is the estimate at :959-982. */
      if (stage == 2 && nana >= 1)
        {
          int cm = 0, c1 = 0, c2 = 0;
          for (int j = 0; j < B1; j++)
            {
              double re = G1[2 * j], im = G1[2 * j + 1];
              if (re * re + im * im > 1e-6)
                c1++;
            }
          for (int j = 0; j < B2; j++)
            {
              double re = G2[2 * j], im = G2[2 * j + 1];
              if (re * re + im * im > 1e-6)
                c2++;
            }
          for (int j = 0; j < W; j++)
            {
              double re = MAN[4 * j] / W, im = MAN[4 * j + 1] / W;
              if (re * re + im * im > 1e-6)
                cm++;
            }
          if (prev_man == cm && prev_g1 == c1 && prev_g2 == c2)
            break;
          prev_man = cm;
          prev_g1 = c1;
          prev_g2 = c2;
        }
      nana++;
      if (nana > V3_MAX_PASSES)
        break;
      stage = (stage + 1) % 3;
    }
  dbg[5] = nana;
  dbg[7] = found;
}

/* ------------------------------------------------------------------ exec -- */

static int tid(void)
{
#ifdef _OPENMP
  return omp_get_thread_num();
#else
  return 0;
#endif
}

typedef struct
{
  int idx;
  double re, im;
} oentry;

static int cmp_entry(const void *x, const void *y)
{
  const oentry *a = (const oentry *)x, *b = (const oentry *)y;
  return (a->idx > b->idx) - (a->idx < b->idx);
}

/* Runs one transform; returns a malloc'd array of distinct entries sorted
 * by frequency (last write wins, as in the dense out[] of the reference). */
static long exec_entries(oracle_plan *p, const double *in, oentry **out)
{
  oscratch *s = &p->scr[tid()];
  oentry *e;
  long cnt = 0;
  if (p->version < 2)
    {
      double *vals;
      o_outer_loop(p, s, in, &vals);
      e = (oentry *)malloc(sizeof(oentry) * (size_t)(s->hits_found + 1));
      for (long i = 0; i < s->hits_found; i++)
        {
          e[i].idx = s->hits[i];
          e[i].re = vals[2 * i];
          e[i].im = vals[2 * i + 1];
        }
      cnt = s->hits_found;
      free(vals);
    }
  else
    {
      omap ans;
      omap_init(&ans);
      o_alternate_fft(p, s, in, &ans);
      e = (oentry *)malloc(sizeof(oentry) * (size_t)(ans.count + 1));
      for (long i = 0; i < ans.count; i++)
        {
          e[i].idx = ans.keys[i];
          e[i].re = ans.vals[2 * i];
          e[i].im = ans.vals[2 * i + 1];
        }
      cnt = ans.count;
      omap_free(&ans);
    }
  /* stable-enough dedupe: entries with one index carry one value */
  qsort(e, cnt, sizeof(oentry), cmp_entry);
  long u = 0;
  for (long i = 0; i < cnt; i++)
    if (u == 0 || e[u - 1].idx != e[i].idx)
      e[u++] = e[i];
  *out = e;
  return u;
}

long oracle_exec(oracle_plan *p, const double *in, int *out_idx, double *out_val, long cap)
{
  if (!p || !in)
    return -1;
  oentry *e;
  long u = exec_entries(p, in, &e);
  if (u > cap)
    {
      free(e);
      return -1;
    }
  for (long i = 0; i < u; i++)
    {
      out_idx[i] = e[i].idx;
      out_val[2 * i] = e[i].re;
      out_val[2 * i + 1] = e[i].im;
    }
  free(e);
  return u;
}

void oracle_exec_many_dense(oracle_plan *p, int num, const double **in, double **out)
{
#pragma omp parallel for schedule(dynamic, 1)
  for (int i = 0; i < num; i++)
    {
      memset(out[i], 0, sizeof(double) * 2 * (size_t)p->n);
      oentry *e;
      long u = exec_entries(p, in[i], &e);
      for (long q = 0; q < u; q++)
        {
          out[i][2 * (long)e[q].idx] = e[q].re;
          out[i][2 * (long)e[q].idx + 1] = e[q].im;
        }
      free(e);
    }
}

/* ----------------------------------------------------------------- debug -- */

const int *oracle_dbg_perm(const oracle_plan *p, int which)
{
  return which ? p->scr[0].ai : p->scr[0].a;
}

const int *oracle_dbg_J(const oracle_plan *p)
{
  return p->scr[0].Jall;
}

const int *oracle_dbg_score(const oracle_plan *p)
{
  return p->scr[0].score;
}

const int *oracle_dbg_hits(const oracle_plan *p, long *count)
{
  *count = p->scr[0].hits_found;
  return p->scr[0].hits;
}

const double *oracle_dbg_xsamp(const oracle_plan *p)
{
  return p->scr[0].x_samp;
}

const int *oracle_dbg_comb(const oracle_plan *p, int *count)
{
  *count = p->scr[0].num_comb;
  return p->scr[0].comb;
}

void oracle_dbg_v3(const oracle_plan *p, int *vals)
{
  memcpy(vals, p->scr[0].v3dbg, sizeof(int) * 8);
}

long oracle_dbg_v3_trace(const oracle_plan *p, double *out, long cap)
{
  long n = p->scr[0].trace_n < p->scr[0].trace_cap ? p->scr[0].trace_n : p->scr[0].trace_cap;
  if (n > cap)
    n = cap;
  memcpy(out, p->scr[0].trace, sizeof(double) * 5 * (size_t)n);
  return n;
}
