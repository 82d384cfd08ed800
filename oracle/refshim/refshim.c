/*
 * refshim.c -- glue that lets the reference's own C sources build and run as the
 * test oracle (oracle/_ref/librsvd_ref.so).  Test infrastructure only: nothing
 * in the product links or loads it.
 *
 *  - VSL replacement (see include/mkl_vsl.h): each vsRngGaussian request is
 *    served by the registered Gaussian-test-matrix provider, so a harness can
 *    hand the reference exactly the sketch matrices it hands the GPU engine.
 *  - LAPACKE_dgeqp3 / LAPACKE_sgeqp3 wrappers that clear jpvt (see include/mkl.h).
 *  - dsecnd (MKL's timer) for the oneAPI variant's sources.
 *  - Thread control for OpenBLAS and OpenMP, for timed CPU baselines.
 *
 * The provider ABI is shared with the port (oracle/port) and the GPU engine
 * (include/rsvdpack.h: rsvdpack_set_omega_provider): the callback fills
 * nrows*ncols doubles in column-major order for request number call_index.
 * The reference only knows the element count of a request, so it asks for
 * (N, 1); a provider must therefore depend on the count, not the shape.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <omp.h>
#include "mkl.h"

typedef void (*rsvd_omega_fn)(void *ctx, int call_index, int nrows, int ncols, double *out);

static rsvd_omega_fn g_provider = NULL;
static void *g_provider_ctx = NULL;
static int g_calls = 0;

void rsvdpack_set_omega_provider(rsvd_omega_fn fn, void *ctx)
{
    g_provider = fn;
    g_provider_ctx = ctx;
    g_calls = 0;
}

void rsvdpack_reset_omega_counter(void) { g_calls = 0; }
int rsvdpack_omega_calls(void) { return g_calls; }

extern void scipy_openblas_set_num_threads(int);

void rsvdpack_set_num_threads(int n)
{
    if (n < 1) n = 1;
    scipy_openblas_set_num_threads(n);
    omp_set_num_threads(n);
}

/* Fallback generator when no provider is registered: splitmix64 counter hash,
 * Box-Muller.  Only needs to be deterministic; it is never compared against. */
static uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static void fallback_gaussians(int call_index, long n, double *out)
{
    for (long i = 0; i < n; i += 2) {
        uint64_t h = mix64(((uint64_t)call_index << 40) ^ (uint64_t)i);
        double u1 = ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        double u2 = ((double)(mix64(h) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        double r = sqrt(-2.0 * log(u1));
        out[i] = r * cos(6.283185307179586 * u2);
        if (i + 1 < n) out[i + 1] = r * sin(6.283185307179586 * u2);
    }
}

int vslNewStream(VSLStreamStatePtr *stream, int brng, unsigned int seed)
{
    (void)brng; (void)seed;
    *stream = NULL;
    return 0;
}

int vslDeleteStream(VSLStreamStatePtr *stream)
{
    *stream = NULL;
    return 0;
}

int vsRngGaussian(int method, VSLStreamStatePtr stream, int n, float *r, float a, float sigma)
{
    (void)method; (void)stream;
    double *tmp = (double *)malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
    if (g_provider) g_provider(g_provider_ctx, g_calls, n, 1, tmp);
    else fallback_gaussians(g_calls, n, tmp);
    g_calls++;
    for (int i = 0; i < n; i++) r[i] = (float)(a + sigma * tmp[i]);
    free(tmp);
    return 0;
}

lapack_int refshim_LAPACKE_dgeqp3(int layout, lapack_int m, lapack_int n, double *a,
                                  lapack_int lda, lapack_int *jpvt, double *tau)
{
    for (lapack_int j = 0; j < n; j++) jpvt[j] = 0;
    return scipy_LAPACKE_dgeqp3(layout, m, n, a, lda, jpvt, tau);
}

lapack_int refshim_LAPACKE_sgeqp3(int layout, lapack_int m, lapack_int n, float *a,
                                  lapack_int lda, lapack_int *jpvt, float *tau)
{
    for (lapack_int j = 0; j < n; j++) jpvt[j] = 0;
    return scipy_LAPACKE_sgeqp3(layout, m, n, a, lda, jpvt, tau);
}

double refshim_seconds(void) { return omp_get_wtime(); }
