// The same from C++, with the reference's sfft_output map type.
#include <cstdio>

#include "sfft.h"

int main() {
  sfft_output out;
  sfft_plan *p = sfft_make_plan(1 << 16, 50, SFFT_VERSION_1, FFTW_ESTIMATE);
  if (!p) {
    std::printf("no plan: %s\n", sfft_last_error());
    return 0;
  }
  complex_t *in = (complex_t *)sfft_malloc((1 << 16) * sizeof(complex_t));
  for (int i = 0; i < (1 << 16); i++) in[i] = 0;
  in[0] = 1;
  sfft_exec_output(p, in, &out);
  std::printf("plan v1 entries=%zu\n", out.size());
  sfft_free(in);
  sfft_free_plan(p);
  return 0;
}
