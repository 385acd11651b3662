/* A C caller written against sFFT 0.1's API (the usage of the reference's
 * test/test.c): plan, page-locked buffers, one dense transform, free.  Prints
 * the plan's status and, with a GPU, the largest output magnitude. */
#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "sfft.h"

int main(void) {
  const int n = 1 << 16, k = 50;
  sfft_plan *p = sfft_make_plan(n, k, SFFT_VERSION_2, FFTW_ESTIMATE);
  if (!p) {
    printf("no plan: %s\n", sfft_last_error());
    return 0;
  }
  complex_t *in = (complex_t *)sfft_malloc(n * sizeof(complex_t));
  complex_t *out = (complex_t *)sfft_malloc(n * sizeof(complex_t));
  for (int i = 0; i < n; i++) in[i] = cexp(2.0 * M_PI * I * (double)(((long)i * 1234) % n) / n);
  sfft_exec(p, in, out);
  double mx = 0;
  for (int i = 0; i < n; i++) mx = fmax(mx, cabs(out[i]));
  printf("plan v%d n=%u k=%u max|out|=%.6f\n", (int)p->version + 1, p->n, p->k, mx);
  sfft_free(in);
  sfft_free(out);
  sfft_free_plan(p);
  return 0;
}
