/*
 * fft_shim.c — FFTW3-subset shim.  TEST INFRASTRUCTURE ONLY: it backs the
 * CPU oracle and the reference build in oracle/_ref; the product never
 * links it.
 *
 * The FFT defined here is THE FFT of this project's parity story: the GPU
 * bucket FFTs and the product's plan-time FFT perform exactly the same
 * IEEE-754 double operations in the same order, so their results are
 * bit-identical to this file's.  The definition:
 *
 *  * Twiddles.  tw[t] = (C(t), -S(t)), t < N, where for N >= 4, Q = N/4,
 *    t = q*Q + u (u < Q): with c = cos(a), s = sin(a),
 *    a = (2.0 * M_PI * u) / N (libm, double):
 *      q=0: (C,S) = ( c,  s)   q=1: (-s,  c)
 *      q=2: (-c, -s)           q=3: ( s, -c)
 *    For N < 4 only tw[0] = (1, -0.0) exists.
 *  * Stages (Stockham autosort).  log2 N odd: one radix-2 stage first
 *    (Ns = 1), then radix-4 stages with Ns = 1 or 2, then x4 each stage.
 *    A stage of radix R reads v[r] = src[j + r*N/R] for j < N/R, r < R;
 *    for r >= 1 and e = r * (j % Ns) * (N / (Ns*R)) != 0 it multiplies
 *    v[r] by tw[e] with re = a*c - b*d, im = a*d + b*c (no fused
 *    multiply-add); then the radix-R butterfly:
 *      R=2: (v0+v1, v0-v1)
 *      R=4: t0=v0+v2 t1=v0-v2 t2=v1+v3 t3=(v1-v3)*(-i)
 *           (t0+t2, t1+t3, t0-t2, t1-t3)
 *    and writes dst[(j - j%Ns)*R + j%Ns + r*Ns] = v[r].
 *  * Backward transform: conj(FFT(conj(x))), unnormalised.
 *  * Lengths that are not powers of two: Bluestein with M = the smallest
 *    power of two >= 2w-1 and chirp ch[m] = (cos(p), -sin(p)),
 *    p = (M_PI * ((m*m) mod 2w)) / w; X[k] = (ch[k] * IFFT_M(FFT_M(a) *
 *    FFT_M(b))[k]) / M with a[m] = x[m]*ch[m], b[m] = b[M-m] = conj(ch[m]).
 *
 * Compile with -ffp-contract=off: contraction into FMA would change bits.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"

/* ---- twiddle tables, cached per length ---------------------------------- */

#define SHIM_MAX_LOG2 31
static double *tw_cache[SHIM_MAX_LOG2 + 1];
static pthread_mutex_t tw_lock = PTHREAD_MUTEX_INITIALIZER;

static int ilog2_exact(long n)
{
  int m = 0;
  while ((1L << m) < n)
    m++;
  return ((1L << m) == n) ? m : -1;
}

static double *make_twiddles(long N)
{
  double *tw = (double *)malloc(sizeof(double) * 2 * (size_t)(N < 1 ? 1 : N));
  if (N < 4)
    {
      tw[0] = 1.0;
      tw[1] = -0.0;
      if (N >= 2)
        {                       /* never read by the stage code, kept defined */
          tw[2] = -1.0;
          tw[3] = -0.0;
        }
      return tw;
    }
  long Q = N / 4;
  for (long u = 0; u < Q; u++)
    {
      double a = (2.0 * M_PI * (double)u) / (double)N;
      double c = cos(a), s = sin(a);
      double C[4] = { c, -s, -c, s };
      double S[4] = { s, c, -s, -c };
      for (int q = 0; q < 4; q++)
        {
          long t = q * Q + u;
          tw[2 * t] = C[q];
          tw[2 * t + 1] = -S[q];
        }
    }
  return tw;
}

const double *shim_twiddles(int n)
{
  int m = ilog2_exact(n);
  if (m < 0)
    return NULL;
  pthread_mutex_lock(&tw_lock);
  if (!tw_cache[m])
    tw_cache[m] = make_twiddles(n);
  double *t = tw_cache[m];
  pthread_mutex_unlock(&tw_lock);
  return t;
}

/* ---- power-of-two Stockham FFT (forward) -------------------------------- */

static inline void cmul_tw(double *re, double *im, const double *w)
{
  double a = *re, b = *im, c = w[0], d = w[1];
  double ac = a * c, bd = b * d, ad = a * d, bc = b * c;
  *re = ac - bd;
  *im = ad + bc;
}

static void fft_pow2_forward(long N, double *a, double *tmp)
{
  if (N <= 1)
    return;
  const double *tw = shim_twiddles((int)N);
  double *src = a, *dst = tmp;
  long Ns = 1;
  int m = ilog2_exact(N);
  if (m & 1)
    {
      long h = N / 2;
      for (long j = 0; j < h; j++)
        {
          double v0r = src[2 * j], v0i = src[2 * j + 1];
          double v1r = src[2 * (j + h)], v1i = src[2 * (j + h) + 1];
          /* Ns == 1: twiddle exponent is 0, no multiply */
          dst[2 * (2 * j)] = v0r + v1r;
          dst[2 * (2 * j) + 1] = v0i + v1i;
          dst[2 * (2 * j + 1)] = v0r - v1r;
          dst[2 * (2 * j + 1) + 1] = v0i - v1i;
        }
      double *t = src;
      src = dst;
      dst = t;
      Ns = 2;
    }
  while (Ns < N)
    {
      long q4 = N / 4;
      long stride = N / (Ns * 4);
      for (long j = 0; j < q4; j++)
        {
          long k = j & (Ns - 1);
          double vr[4], vi[4];
          for (int r = 0; r < 4; r++)
            {
              vr[r] = src[2 * (j + r * q4)];
              vi[r] = src[2 * (j + r * q4) + 1];
            }
          for (int r = 1; r < 4; r++)
            {
              long e = (long)r * k * stride;
              if (e)
                cmul_tw(&vr[r], &vi[r], tw + 2 * e);
            }
          double t0r = vr[0] + vr[2], t0i = vi[0] + vi[2];
          double t1r = vr[0] - vr[2], t1i = vi[0] - vi[2];
          double t2r = vr[1] + vr[3], t2i = vi[1] + vi[3];
          double t3r = vr[1] - vr[3], t3i = vi[1] - vi[3];
          /* t3 *= -i */
          double u3r = t3i, u3i = -t3r;
          long base = (j - k) * 4 + k;
          dst[2 * base] = t0r + t2r;
          dst[2 * base + 1] = t0i + t2i;
          dst[2 * (base + Ns)] = t1r + u3r;
          dst[2 * (base + Ns) + 1] = t1i + u3i;
          dst[2 * (base + 2 * Ns)] = t0r - t2r;
          dst[2 * (base + 2 * Ns) + 1] = t0i - t2i;
          dst[2 * (base + 3 * Ns)] = t1r - u3r;
          dst[2 * (base + 3 * Ns) + 1] = t1i - u3i;
        }
      double *t = src;
      src = dst;
      dst = t;
      Ns *= 4;
    }
  if (src != a)
    memcpy(a, src, sizeof(double) * 2 * (size_t)N);
}

static void conj_inplace(long n, double *a)
{
  for (long i = 0; i < n; i++)
    a[2 * i + 1] = -a[2 * i + 1];
}

static void fft_pow2(long N, double *a, int sign)
{
  double *tmp = (double *)malloc(sizeof(double) * 2 * (size_t)N);
  if (sign > 0)
    conj_inplace(N, a);
  fft_pow2_forward(N, a, tmp);
  if (sign > 0)
    conj_inplace(N, a);
  free(tmp);
}

/* ---- Bluestein for any other length ------------------------------------- */

static void fft_bluestein(long w, double *x, int sign)
{
  long M = 1;
  while (M < 2 * w - 1)
    M <<= 1;
  double *ch = (double *)malloc(sizeof(double) * 2 * (size_t)w);
  double *A = (double *)calloc(2 * (size_t)M, sizeof(double));
  double *Bv = (double *)calloc(2 * (size_t)M, sizeof(double));
  for (long m = 0; m < w; m++)
    {
      long e = (long)(((uint64_t)m * (uint64_t)m) % (uint64_t)(2 * w));
      double p = (M_PI * (double)e) / (double)w;
      ch[2 * m] = cos(p);
      ch[2 * m + 1] = -sin(p);
    }
  if (sign > 0)
    conj_inplace(w, x);
  for (long m = 0; m < w; m++)
    {
      double re = x[2 * m], im = x[2 * m + 1];
      cmul_tw(&re, &im, ch + 2 * m);
      A[2 * m] = re;
      A[2 * m + 1] = im;
      Bv[2 * m] = ch[2 * m];
      Bv[2 * m + 1] = -ch[2 * m + 1];
      if (m)
        {
          Bv[2 * (M - m)] = ch[2 * m];
          Bv[2 * (M - m) + 1] = -ch[2 * m + 1];
        }
    }
  fft_pow2(M, A, -1);
  fft_pow2(M, Bv, -1);
  for (long i = 0; i < M; i++)
    {
      double re = A[2 * i], im = A[2 * i + 1];
      cmul_tw(&re, &im, Bv + 2 * i);
      A[2 * i] = re;
      A[2 * i + 1] = im;
    }
  fft_pow2(M, A, +1);
  for (long kk = 0; kk < w; kk++)
    {
      double re = A[2 * kk], im = A[2 * kk + 1];
      cmul_tw(&re, &im, ch + 2 * kk);
      x[2 * kk] = re / (double)M;
      x[2 * kk + 1] = im / (double)M;
    }
  if (sign > 0)
    conj_inplace(w, x);
  free(ch);
  free(A);
  free(Bv);
}

void shim_fft(int n, double *data, int sign)
{
  if (n <= 1)
    return;
  if (ilog2_exact(n) >= 0)
    fft_pow2(n, data, sign);
  else
    fft_bluestein(n, data, sign);
}

/* ---- the FFTW plan interface -------------------------------------------- */

struct shim_fft_plan
{
  int n, howmany, istride, idist, ostride, odist, sign;
  double *in, *out;
};

fftw_plan fftw_plan_many_dft(int rank, const int *n, int howmany,
                             fftw_complex *in, const int *inembed,
                             int istride, int idist,
                             fftw_complex *out, const int *onembed,
                             int ostride, int odist, int sign, unsigned flags)
{
  (void)inembed;
  (void)onembed;
  (void)flags;
  if (rank != 1 || howmany < 1)
    return NULL;
  /* the reference passes one size per transform; they are all equal */
  for (int i = 1; i < howmany; i++)
    if (n[i] != n[0])
      return NULL;
  struct shim_fft_plan *p = (struct shim_fft_plan *)calloc(1, sizeof(*p));
  p->n = n[0];
  p->howmany = howmany;
  p->in = (double *)in;
  p->out = (double *)out;
  p->istride = istride;
  p->idist = idist;
  p->ostride = ostride;
  p->odist = odist;
  p->sign = sign;
  return p;
}

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out,
                           int sign, unsigned flags)
{
  return fftw_plan_many_dft(1, &n, 1, in, NULL, 1, n, out, NULL, 1, n,
                            sign, flags);
}

void fftw_execute(const fftw_plan p)
{
  if (!p)
    return;
  double *buf = (double *)malloc(sizeof(double) * 2 * (size_t)p->n);
  for (int t = 0; t < p->howmany; t++)
    {
      const double *src = p->in + 2 * (size_t)t * p->idist;
      for (int i = 0; i < p->n; i++)
        {
          buf[2 * i] = src[2 * (size_t)i * p->istride];
          buf[2 * i + 1] = src[2 * (size_t)i * p->istride + 1];
        }
      shim_fft(p->n, buf, p->sign);
      double *dst = p->out + 2 * (size_t)t * p->odist;
      for (int i = 0; i < p->n; i++)
        {
          dst[2 * (size_t)i * p->ostride] = buf[2 * i];
          dst[2 * (size_t)i * p->ostride + 1] = buf[2 * i + 1];
        }
    }
  free(buf);
}

void fftw_destroy_plan(fftw_plan p)
{
  free(p);
}

void *fftw_malloc(size_t n)
{
  void *q = NULL;
  if (posix_memalign(&q, 64, n ? n : 1))
    return NULL;
  return q;
}

void fftw_free(void *p)
{
  free(p);
}

/* Flop model used by the reference's optional counters: 5 N log2 N. */
void fftw_flops(const fftw_plan p, double *add, double *mul, double *fma)
{
  double n = p ? p->n : 0, h = p ? p->howmany : 0;
  double f = n > 1 ? 5.0 * n * log2(n) * h : 0.0;
  *add = 0.6 * f;
  *mul = 0.4 * f;
  *fma = 0.0;
}
