/*
 * Stand-in for MKL VSL, used ONLY to compile the reference's sources into the
 * test oracle.  The reference draws every Gaussian test matrix with
 * vslNewStream(MCG31, time(NULL)) + vsRngGaussian(ICDF) in float
 * (multi_core_mkl_code/matrix_vector_functions_intel_mkl.c:458-486), so its runs
 * are not repeatable.  Here each vsRngGaussian request is served by a provider
 * the harness registers (refshim_set_omega_provider in refshim.c): request
 * number c (0-based, counted per process) of N floats is filled in the order the
 * reference stores them, i.e. the column-major entries of the matrix being
 * initialised.  With no provider, a fixed counter-based generator is used.
 */
#ifndef RSVD_REFSHIM_MKL_VSL_H
#define RSVD_REFSHIM_MKL_VSL_H

#ifdef __cplusplus
extern "C" {
#endif

typedef void *VSLStreamStatePtr;
#define VSL_BRNG_MCG31 1
#define VSL_RNG_METHOD_GAUSSIAN_ICDF 2

int vslNewStream(VSLStreamStatePtr *stream, int brng, unsigned int seed);
int vslDeleteStream(VSLStreamStatePtr *stream);
int vsRngGaussian(int method, VSLStreamStatePtr stream, int n, float *r, float a, float sigma);

#ifdef __cplusplus
}
#endif

#endif
