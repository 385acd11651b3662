/*
 * ref_pad.c — linked only into oracle/_ref (the unmodified reference built
 * against the FFT shim).  TEST INFRASTRUCTURE.
 *
 * The reference writes one element past its v3 `perm_x` buffer
 * (src/sfft.cc:497-498 allocate w_g2 elements, src/computefourier-3.0.cc:
 * 235-236 write w_g2 + 1).  Every aligned allocation it makes goes through
 * posix_memalign (_mm_malloc); the link wraps that call and pads each
 * block by 64 bytes so the extra element lands in owned memory.
 */
#include <stddef.h>

int __real_posix_memalign(void **p, size_t align, size_t size);

int __wrap_posix_memalign(void **p, size_t align, size_t size)
{
  return __real_posix_memalign(p, align, size + 64);
}
