/*
 * Stand-in for Intel MKL's umbrella header, used ONLY to compile the reference's
 * own C sources (multi_core_mkl_code/rank_revealing_algorithms_intel_mkl.c and
 * multi_core_mkl_code/matrix_vector_functions_intel_mkl.c) into the test oracle
 * oracle/_ref/librsvd_ref.so.  Test infrastructure, never shipped.
 *
 * The reference calls MKL's CBLAS/LAPACKE/VSL entry points.  MKL is absent here;
 * scipy's bundled OpenBLAS exports the same CBLAS/LAPACKE routines with a
 * "scipy_" prefix (LP64, 32-bit int).  This header maps each name the reference
 * uses onto that prefix.  VSL is replaced by refshim.c (see mkl_vsl.h).
 */
#ifndef RSVD_REFSHIM_MKL_H
#define RSVD_REFSHIM_MKL_H

#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <omp.h>   /* the oneAPI variant's sources call omp_get_wtime without including it */

#ifdef __cplusplus
extern "C" {
#endif

/* CBLAS enumerations: values are fixed by the CBLAS standard. */
typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_LAYOUT;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;
typedef enum { CblasUpper = 121, CblasLower = 122 } CBLAS_UPLO;
typedef enum { CblasNonUnit = 131, CblasUnit = 132 } CBLAS_DIAG;
typedef enum { CblasLeft = 141, CblasRight = 142 } CBLAS_SIDE;

#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
typedef int lapack_int;

void scipy_cblas_dgemm(int layout, int transa, int transb, int m, int n, int k,
                       double alpha, const double *a, int lda, const double *b, int ldb,
                       double beta, double *c, int ldc);
void scipy_cblas_dgemv(int layout, int trans, int m, int n, double alpha,
                       const double *a, int lda, const double *x, int incx,
                       double beta, double *y, int incy);
void scipy_cblas_dtrsm(int layout, int side, int uplo, int transa, int diag,
                       int m, int n, double alpha, const double *a, int lda,
                       double *b, int ldb);
void scipy_cblas_dtrsv(int layout, int uplo, int trans, int diag, int n,
                       const double *a, int lda, double *x, int incx);

lapack_int scipy_LAPACKE_dgeqrf(int layout, lapack_int m, lapack_int n, double *a,
                                lapack_int lda, double *tau);
lapack_int scipy_LAPACKE_dorgqr(int layout, lapack_int m, lapack_int n, lapack_int k,
                                double *a, lapack_int lda, const double *tau);
lapack_int scipy_LAPACKE_dgeqp3(int layout, lapack_int m, lapack_int n, double *a,
                                lapack_int lda, lapack_int *jpvt, double *tau);
lapack_int scipy_LAPACKE_dgesvd(int layout, char jobu, char jobvt, lapack_int m,
                                lapack_int n, double *a, lapack_int lda, double *s,
                                double *u, lapack_int ldu, double *vt, lapack_int ldvt,
                                double *superb);
lapack_int scipy_LAPACKE_dsyev(int layout, char jobz, char uplo, lapack_int n,
                               double *a, lapack_int lda, double *w);
lapack_int scipy_LAPACKE_dtrtri(int layout, char uplo, char diag, lapack_int n,
                                double *a, lapack_int lda);
lapack_int scipy_LAPACKE_dgesv(int layout, lapack_int n, lapack_int nrhs, double *a,
                               lapack_int lda, lapack_int *ipiv, double *b, lapack_int ldb);

/* dgeqp3 treats a nonzero jpvt(j) as "column j is fixed in front".  The
 * reference passes a malloc'd, uninitialised jpvt (rank_revealing_algorithms_intel_mkl.c:934,947),
 * so its pivots are undefined.  The oracle defines them: refshim.c clears jpvt
 * before the call, i.e. every column is free. */
lapack_int refshim_LAPACKE_dgeqp3(int layout, lapack_int m, lapack_int n, double *a,
                                  lapack_int lda, lapack_int *jpvt, double *tau);

#define cblas_dgemm   scipy_cblas_dgemm
#define cblas_dgemv   scipy_cblas_dgemv
#define cblas_dtrsm   scipy_cblas_dtrsm
#define cblas_dtrsv   scipy_cblas_dtrsv
#define LAPACKE_dgeqrf scipy_LAPACKE_dgeqrf
#define LAPACKE_dorgqr scipy_LAPACKE_dorgqr
#define LAPACKE_dgeqp3 refshim_LAPACKE_dgeqp3
#define LAPACKE_dgesvd scipy_LAPACKE_dgesvd
#define LAPACKE_dsyev  scipy_LAPACKE_dsyev
#define LAPACKE_dtrtri scipy_LAPACKE_dtrtri
#define LAPACKE_dgesv  scipy_LAPACKE_dgesv

/* Single precision and MKL service calls, used by the oneAPI variant's sources
 * (oneapi_code/matrix_vector_functions_one_api.c, rank_revealing_algorithms_one_api.c),
 * compiled into oracle/_ref/librsvd_ref_f32.so the same way. */
void scipy_cblas_sgemm(int layout, int transa, int transb, int m, int n, int k,
                       float alpha, const float *a, int lda, const float *b, int ldb,
                       float beta, float *c, int ldc);
void scipy_cblas_sgemv(int layout, int trans, int m, int n, float alpha,
                       const float *a, int lda, const float *x, int incx,
                       float beta, float *y, int incy);
void scipy_cblas_strsm(int layout, int side, int uplo, int transa, int diag,
                       int m, int n, float alpha, const float *a, int lda,
                       float *b, int ldb);
void scipy_cblas_strsv(int layout, int uplo, int trans, int diag, int n,
                       const float *a, int lda, float *x, int incx);
lapack_int scipy_LAPACKE_sgeqrf(int layout, lapack_int m, lapack_int n, float *a,
                                lapack_int lda, float *tau);
lapack_int scipy_LAPACKE_sorgqr(int layout, lapack_int m, lapack_int n, lapack_int k,
                                float *a, lapack_int lda, const float *tau);
lapack_int scipy_LAPACKE_sgeqp3(int layout, lapack_int m, lapack_int n, float *a,
                                lapack_int lda, lapack_int *jpvt, float *tau);
lapack_int scipy_LAPACKE_sgesvd(int layout, char jobu, char jobvt, lapack_int m,
                                lapack_int n, float *a, lapack_int lda, float *s,
                                float *u, lapack_int ldu, float *vt, lapack_int ldvt,
                                float *superb);
lapack_int scipy_LAPACKE_ssyev(int layout, char jobz, char uplo, lapack_int n,
                               float *a, lapack_int lda, float *w);
lapack_int scipy_LAPACKE_sgesv(int layout, lapack_int n, lapack_int nrhs, float *a,
                               lapack_int lda, lapack_int *ipiv, float *b, lapack_int ldb);
/* the oneAPI pivotedQR_mkl passes an uninitialised jpvt too (one_api.c:830,844) */
lapack_int refshim_LAPACKE_sgeqp3(int layout, lapack_int m, lapack_int n, float *a,
                                  lapack_int lda, lapack_int *jpvt, float *tau);

#define cblas_sgemm    scipy_cblas_sgemm
#define cblas_sgemv    scipy_cblas_sgemv
#define cblas_strsm    scipy_cblas_strsm
#define cblas_strsv    scipy_cblas_strsv
#define LAPACKE_sgeqrf scipy_LAPACKE_sgeqrf
#define LAPACKE_sorgqr scipy_LAPACKE_sorgqr
#define LAPACKE_sgeqp3 refshim_LAPACKE_sgeqp3
#define LAPACKE_sgesvd scipy_LAPACKE_sgesvd
#define LAPACKE_ssyev  scipy_LAPACKE_ssyev
#define LAPACKE_sgesv  scipy_LAPACKE_sgesv

/* MKL service functions: aligned allocation (calloc'd, as the reference relies on zeroed
 * matrices) and the wall-clock timer */
static inline void *mkl_calloc(size_t num, size_t size, int alignment)
{
    (void)alignment;
    return calloc(num ? num : 1, size);
}
static inline void mkl_free(void *p) { free(p); }
double refshim_seconds(void);
#define dsecnd refshim_seconds

#ifdef __cplusplus
}
#endif

#include "mkl_vsl.h"

#endif
