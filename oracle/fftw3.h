/*
 * fftw3.h — interface of the FFTW3 subset that the sFFT 0.1 sources call.
 *
 * TEST INFRASTRUCTURE.  FFTW itself is not available here, so this header
 * and fft_shim.c stand in for it when the oracle (and the unmodified
 * reference, built into oracle/_ref) are compiled.  Only the names,
 * argument meanings and sign conventions of FFTW 3 are kept
 * (FFTW_FORWARD = e^{-2 pi i jk/n}, FFTW_BACKWARD unnormalised); the
 * arithmetic is this project's own radix-4/2 Stockham FFT (Bluestein for
 * lengths that are not powers of two), described in fft_shim.c.
 *
 * Reference call sites: src/fftw.cc:29-59, src/sfft.cc:255-296 and
 * :422-477, src/computefourier-1.0-2.0.cc:69,270,273,
 * src/computefourier-3.0.cc:123,208,293.
 */
#ifndef SFFT_SHIM_FFTW3_H
#define SFFT_SHIM_FFTW3_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* FFTW makes fftw_complex a C99 complex when <complex.h> is in scope;
 * the reference relies on that (src/fft.h:42-45), so it is always so here. */
typedef double _Complex fftw_complex;

typedef struct shim_fft_plan *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out,
                           int sign, unsigned flags);
fftw_plan fftw_plan_many_dft(int rank, const int *n, int howmany,
                             fftw_complex *in, const int *inembed,
                             int istride, int idist,
                             fftw_complex *out, const int *onembed,
                             int ostride, int odist,
                             int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
void *fftw_malloc(size_t n);
void fftw_free(void *p);
void fftw_flops(const fftw_plan p, double *add, double *mul, double *fma);

/* Direct entry points of the shim (used by the oracle restatement).
 * data: n interleaved (re, im) doubles, transformed in place.
 * sign: -1 forward, +1 backward (unnormalised). */
void shim_fft(int n, double *data, int sign);
/* Twiddle table of the power-of-two FFT: tw[2t], tw[2t+1] for t < n. */
const double *shim_twiddles(int n);

#ifdef __cplusplus
}
#endif

#endif
