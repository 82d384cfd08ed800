/*
 * Drop-in stand-in for oneapi_code/rank_revealing_algorithms_one_api.h: a caller of that variant compiles unchanged with
 * -I include/compat/oneapi -I include and links librsvdpack_f32.so.  Declarations: rsvdpack.h.
 */
#ifndef RSVDPACK_COMPAT_ONEAPI_RANK_REVEALING_ALGORITHMS_ONE_API_H
#define RSVDPACK_COMPAT_ONEAPI_RANK_REVEALING_ALGORITHMS_ONE_API_H

#ifndef RSVDPACK_REAL32
#define RSVDPACK_REAL32
#endif
#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>
#include <inttypes.h>
#include <math.h>
#include <time.h>
#include <sys/time.h>
#include "rsvdpack.h"

/* MKL's wall-clock timer, which the reference's drivers call (MKL is replaced on the link line) */
#ifndef RSVDPACK_COMPAT_DSECND
#define RSVDPACK_COMPAT_DSECND
static inline double dsecnd(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}
#endif

/* the convenience macros the reference's header defines */
#ifndef min
#define min(x, y) (((x) < (y)) ? (x) : (y))
#endif
#ifndef max
#define max(x, y) (((x) > (y)) ? (x) : (y))
#endif

/* the index type the oneAPI variant's callers declare (matrix_vector_functions_one_api.h:20) */
#ifndef RSVDPACK_COMPAT_MYINT64
#define RSVDPACK_COMPAT_MYINT64
typedef int64_t myint64;
#endif

#endif
