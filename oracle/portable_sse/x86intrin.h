/* x86intrin.h stand-in for building the sFFT 0.1 reference (checker only)
 * on hosts without x86 SSE, e.g. the aarch64 host of the GPU.
 *
 * The reference's src/intrinsics.h includes <x86intrin.h>; its kernels use
 * 17 SSE2/SSE3 double-precision intrinsics on __m128d.  Each is defined
 * here by its documented lane semantics with GCC vector extensions, so
 * every lane performs the same single IEEE-754 operation as the x86
 * instruction.  The oracle Makefile puts this directory first on the
 * include path only when the host is not x86-64; on x86-64 the compiler's
 * own header is used.  Test infrastructure, never part of the library. */
#ifndef SFFT_PORTABLE_X86INTRIN_H
#define SFFT_PORTABLE_X86INTRIN_H

#include <stdlib.h>

typedef double __m128d __attribute__((vector_size(16), aligned(16)));

#define SFFT_SSE_INLINE static inline __attribute__((always_inline))

/* construction */
SFFT_SSE_INLINE __m128d _mm_set_pd(double hi, double lo) { __m128d r = {lo, hi}; return r; }
SFFT_SSE_INLINE __m128d _mm_set1_pd(double v) { __m128d r = {v, v}; return r; }

/* aligned loads and stores (the address is 16-byte aligned, as on x86) */
SFFT_SSE_INLINE __m128d _mm_load_pd(const double *p) { return *(const __m128d *)p; }
SFFT_SSE_INLINE void _mm_store_pd(double *p, __m128d v) { *(__m128d *)p = v; }
SFFT_SSE_INLINE void _mm_storel_pd(double *p, __m128d v) { *p = v[0]; }
SFFT_SSE_INLINE void _mm_storeh_pd(double *p, __m128d v) { *p = v[1]; }

/* lane-wise arithmetic */
SFFT_SSE_INLINE __m128d _mm_add_pd(__m128d a, __m128d b) { return a + b; }
SFFT_SSE_INLINE __m128d _mm_sub_pd(__m128d a, __m128d b) { return a - b; }
SFFT_SSE_INLINE __m128d _mm_mul_pd(__m128d a, __m128d b) { return a * b; }
SFFT_SSE_INLINE __m128d _mm_div_pd(__m128d a, __m128d b) { return a / b; }

/* horizontal add (SSE3): (a0 + a1, b0 + b1) */
SFFT_SSE_INLINE __m128d _mm_hadd_pd(__m128d a, __m128d b) {
  __m128d r = {a[0] + a[1], b[0] + b[1]};
  return r;
}
/* alternating subtract / add (SSE3): (a0 - b0, a1 + b1) */
SFFT_SSE_INLINE __m128d _mm_addsub_pd(__m128d a, __m128d b) {
  __m128d r = {a[0] - b[0], a[1] + b[1]};
  return r;
}

/* lane selection: bit 0 of imm picks a's lane, bit 1 b's lane */
#define _mm_shuffle_pd(a, b, imm) \
  (__extension__({ __m128d a_ = (a), b_ = (b); __m128d r_ = {a_[(imm) & 1], b_[((imm) >> 1) & 1]}; r_; }))
SFFT_SSE_INLINE __m128d _mm_unpacklo_pd(__m128d a, __m128d b) { __m128d r = {a[0], b[0]}; return r; }
SFFT_SSE_INLINE __m128d _mm_unpackhi_pd(__m128d a, __m128d b) { __m128d r = {a[1], b[1]}; return r; }

/* aligned allocation */
SFFT_SSE_INLINE void *_mm_malloc(size_t size, size_t align) {
  void *p = NULL;
  if (align < sizeof(void *)) align = sizeof(void *);
  return posix_memalign(&p, align, size) == 0 ? p : NULL;
}
SFFT_SSE_INLINE void _mm_free(void *p) { free(p); }

#endif
