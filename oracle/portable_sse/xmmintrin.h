/* xmmintrin.h stand-in: the same definitions as x86intrin.h here. */
#include "x86intrin.h"
