/*
 * Drop-in stand-in for multi_core_mkl_code/matrix_vector_functions_intel_mkl.h: a caller of that variant compiles unchanged with
 * -I include/compat/mkl -I include and links librsvdpack.so.  Declarations: rsvdpack.h.
 */
#ifndef RSVDPACK_COMPAT_MKL_MATRIX_VECTOR_FUNCTIONS_INTEL_MKL_H
#define RSVDPACK_COMPAT_MKL_MATRIX_VECTOR_FUNCTIONS_INTEL_MKL_H

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

#endif
