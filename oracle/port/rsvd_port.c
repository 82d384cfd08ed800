/*
 * rsvd_port.c -- TEST ORACLE (test infrastructure, never the product).
 *
 * A CPU restatement, in our own code, of RSVDPACK's hot-path algorithms from
 * multi_core_mkl_code/rank_revealing_algorithms_intel_mkl.c ("RRA") and the
 * helpers they use in multi_core_mkl_code/matrix_vector_functions_intel_mkl.c
 * ("MVF").  Each routine cites the reference lines it follows.  It issues the
 * same LAPACK/CBLAS calls in the same order with the same arguments, so on the
 * same OpenBLAS it reproduces the reference build (oracle/_ref) bit for bit;
 * that is checked by tests/test_oracle_pin.py and by the committed golden
 * fixtures in tests/golden/.  The reference's semantic quirks are kept on
 * purpose (q-1 power iterations in the fixed-rank SVD, ascending singular
 * values for vnum==2, absolute TOL, floor((k+p)/kstep), even-step
 * re-orthogonalisation, ...), because the GPU engine must reproduce them.
 *
 * Differences from the reference that do not change results:
 *  - no progress printf()s;
 *  - Frobenius norms are summed serially (the reference sums with an OpenMP
 *    reduction, whose rounding depends on the thread count);
 *  - dgeqp3's jpvt is cleared before the call (the reference passes it
 *    uninitialised; cleared is the only defined reading).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>
#include "rsvd_port.h"

/* ---- CBLAS / LAPACKE from scipy's OpenBLAS (LP64, "scipy_" prefix) ---- */
enum { COLMAJ = 102, NOTR = 111, TR = 112, UPPER = 121, NONUNIT = 131, LEFT = 141 };
void scipy_cblas_dgemm(int, int, int, int, int, int, double, const double *, int,
                       const double *, int, double, double *, int);
void scipy_cblas_dtrsm(int, int, int, int, int, int, int, double, const double *, int,
                       double *, int);
int scipy_LAPACKE_dgeqrf(int, int, int, double *, int, double *);
int scipy_LAPACKE_dorgqr(int, int, int, int, double *, int, const double *);
int scipy_LAPACKE_dgeqp3(int, int, int, double *, int, int *, double *);
int scipy_LAPACKE_dgesvd(int, char, char, int, int, double *, int, double *, double *, int,
                         double *, int, double *);
int scipy_LAPACKE_dsyev(int, char, char, int, double *, int, double *);
int scipy_LAPACKE_dgesv(int, int, int, double *, int, int *, double *, int);
void scipy_openblas_set_num_threads(int);

#define MIN(a, b) ((a) < (b) ? (a) : (b))
#define AT(M, i, j) ((M)->d[(size_t)(j) * (size_t)(M)->nrows + (size_t)(i)])

/* ===================== storage (MVF:8-43) ===================== */
mat *matrix_new(int nrows, int ncols)
{
    mat *M = (mat *)malloc(sizeof(mat));
    M->nrows = nrows;
    M->ncols = ncols;
    M->d = (double *)calloc((size_t)nrows * (size_t)ncols, sizeof(double));
    return M;
}

vec *vector_new(int nrows)
{
    vec *v = (vec *)malloc(sizeof(vec));
    v->nrows = nrows;
    v->d = (double *)calloc((size_t)nrows, sizeof(double));
    return v;
}

void matrix_delete(mat *M) { if (M) { free(M->d); free(M); } }
void vector_delete(vec *v) { if (v) { free(v->d); free(v); } }

static size_t nel(const mat *M) { return (size_t)M->nrows * (size_t)M->ncols; }
static mat *dup(const mat *M)
{
    mat *D = matrix_new(M->nrows, M->ncols);
    memcpy(D->d, M->d, nel(M) * sizeof(double));
    return D;
}

/* ===================== Gaussian test matrices (MVF:458-486) ===================== */
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
void rsvdpack_set_num_threads(int n)
{
    if (n < 1) n = 1;
    scipy_openblas_set_num_threads(n);
    omp_set_num_threads(n);
}

static uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* The reference draws floats and widens them to double; a provider is asked for
 * the column-major entries of M.  Values are rounded through float exactly as
 * the reference's float buffer would round them. */
void initialize_random_matrix(mat *M)
{
    size_t n = nel(M);
    if (g_provider) {
        g_provider(g_provider_ctx, g_calls, M->nrows, M->ncols, M->d);
    } else {
        for (size_t i = 0; i < n; i += 2) {
            uint64_t h = mix64(((uint64_t)g_calls << 40) ^ (uint64_t)i);
            double u1 = ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
            double u2 = ((double)(mix64(h) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
            double r = sqrt(-2.0 * log(u1));
            M->d[i] = r * cos(6.283185307179586 * u2);
            if (i + 1 < n) M->d[i + 1] = r * sin(6.283185307179586 * u2);
        }
    }
    for (size_t i = 0; i < n; i++) M->d[i] = (double)(float)M->d[i];
    g_calls++;
}

/* ===================== dense kernels (MVF:538-561, 1214-1284, 1206, 1477-1531) ===================== */
/* C = A*B */
static void gemm_nn(const mat *A, const mat *B, mat *C)
{
    scipy_cblas_dgemm(COLMAJ, NOTR, NOTR, A->nrows, B->ncols, A->ncols, 1.0, A->d, A->nrows,
                      B->d, B->nrows, 0.0, C->d, C->nrows);
}
/* C = A^T*B */
static void gemm_tn(const mat *A, const mat *B, mat *C)
{
    scipy_cblas_dgemm(COLMAJ, TR, NOTR, A->ncols, B->ncols, A->nrows, 1.0, A->d, A->nrows,
                      B->d, B->nrows, 0.0, C->d, C->nrows);
}
/* C = A*B^T */
static void gemm_nt(const mat *A, const mat *B, mat *C)
{
    scipy_cblas_dgemm(COLMAJ, NOTR, TR, A->nrows, B->nrows, A->ncols, 1.0, A->d, A->nrows,
                      B->d, B->nrows, 0.0, C->d, C->nrows);
}

/* Q = orth(Y) through dgeqrf + dorgqr (MVF:1251-1263). */
static void orth_q(const mat *Y, mat *Q)
{
    int m = Y->nrows, n = Y->ncols;
    double *tau = (double *)calloc((size_t)MIN(m, n), sizeof(double));
    memcpy(Q->d, Y->d, nel(Y) * sizeof(double));
    scipy_LAPACKE_dgeqrf(COLMAJ, m, n, Q->d, m, tau);
    scipy_LAPACKE_dorgqr(COLMAJ, m, n, n, Q->d, m, tau);
    free(tau);
}

/* [Q,R] = qr(M,0) (MVF:1214-1245). */
static void qr_econ(const mat *M, mat *Q, mat *R)
{
    int m = M->nrows, n = M->ncols, k = MIN(m, n);
    mat *W = dup(M);
    double *tau = (double *)calloc((size_t)k, sizeof(double));
    scipy_LAPACKE_dgeqrf(COLMAJ, m, n, W->d, m, tau);
    for (int j = 0; j < k; j++)
        for (int i = 0; i <= j; i++) AT(R, i, j) = AT(W, i, j);
    memcpy(Q->d, W->d, nel(W) * sizeof(double));
    scipy_LAPACKE_dorgqr(COLMAJ, Q->nrows, Q->ncols, MIN(Q->ncols, Q->nrows), Q->d, Q->nrows, tau);
    free(tau);
    matrix_delete(W);
}

/* M = U*diag(s)*Vt by dgesvd('S','S'); S receives diag(s); M is overwritten (MVF:1270-1284). */
static void svd_small(mat *M, mat *U, mat *S, mat *Vt)
{
    int m = M->nrows, n = M->ncols, k = MIN(m, n);
    double *s = (double *)calloc((size_t)k, sizeof(double));
    double *superb = (double *)calloc((size_t)(k + 1), sizeof(double));
    scipy_LAPACKE_dgesvd(COLMAJ, 'S', 'S', m, n, M->d, m, s, U->d, m, Vt->d, k, superb);
    for (int i = 0; i < S->nrows && i < k; i++) AT(S, i, i) = s[i];
    free(s);
    free(superb);
}

/* X = triu(A)^{-1} B by dtrsm (MVF:1477-1493, solve_type 1). */
static void tri_solve(const mat *A, const mat *B, mat *X)
{
    memcpy(X->d, B->d, nel(B) * sizeof(double));
    scipy_cblas_dtrsm(COLMAJ, LEFT, UPPER, NOTR, NONUNIT, B->nrows, B->ncols, 1.0, A->d,
                      A->nrows, X->d, X->nrows);
}

static double frob(const mat *M)
{
    double acc = 0.0;
    size_t n = nel(M);
    for (size_t i = 0; i < n; i++) acc += M->d[i] * M->d[i];
    return sqrt(acc);
}

double get_matrix_frobenius_norm(mat *M) { return frob(M); }

double get_percent_error_between_two_mats(mat *A, mat *B)
{
    double num = 0.0;
    size_t n = nel(A);
    for (size_t i = 0; i < n; i++) {
        double d = A->d[i] - B->d[i];
        num += d * d;
    }
    return 100.0 * sqrt(num) / frob(A);
}

void form_svd_product_matrix(mat *U, mat *S, mat *V, mat *P)
{
    mat *SVt = matrix_new(S->nrows, P->ncols);
    gemm_nt(S, V, SVt);
    gemm_nn(U, SVt, P);
    matrix_delete(SVt);
}

void form_cur_product_matrix(mat *C, mat *U, mat *R, mat *P)
{
    mat *CU = matrix_new(P->nrows, U->nrows);
    gemm_nn(C, U, CU);
    gemm_nn(CU, R, P);
    matrix_delete(CU);
}

/* column / row slices (MVF:1078-1128 resize_*, 975-1008 fill_*) */
static mat *cols(const mat *M, int c0, int nc)
{
    mat *R = matrix_new(M->nrows, nc);
    memcpy(R->d, M->d + (size_t)c0 * M->nrows, (size_t)nc * M->nrows * sizeof(double));
    return R;
}
static mat *rows(const mat *M, int r0, int nr)
{
    mat *R = matrix_new(nr, M->ncols);
    for (int j = 0; j < M->ncols; j++)
        for (int i = 0; i < nr; i++) AT(R, i, j) = AT(M, r0 + i, j);
    return R;
}
static mat *block(const mat *M, int r0, int nr, int c0, int nc)
{
    mat *R = matrix_new(nr, nc);
    for (int j = 0; j < nc; j++)
        for (int i = 0; i < nr; i++) AT(R, i, j) = AT(M, r0 + i, c0 + j);
    return R;
}
static mat *transpose(const mat *M)
{
    mat *T = matrix_new(M->ncols, M->nrows);
    for (int j = 0; j < M->ncols; j++)
        for (int i = 0; i < M->nrows; i++) AT(T, j, i) = AT(M, i, j);
    return T;
}
static void replace(mat **dst, mat *src) { matrix_delete(*dst); *dst = src; }

/* ===================== SVD back end shared by the two rSVD drivers ===================== */
/* Given Q (m x l) spanning the sketch, form U,S,V as RRA:133-224 do (vnum 1 / 2)
 * and truncate to rank k (from the front for vnum 1, from the back for vnum 2). */
static void svd_from_q(mat *M, mat *Q, int k, int vnum, mat **U, mat **S, mat **V)
{
    int m = M->nrows, n = M->ncols, l = Q->ncols;
    *U = matrix_new(m, l);
    *S = matrix_new(l, l);
    *V = matrix_new(n, l);
    if (vnum == 1 || vnum > 2) {
        /* RRA:133-174 : Bt = M^T Q ; [Qh,Rh] = qr(Bt) ; [Uh,S,Vh^T] = svd(Rh) ; U = Q Vh ; V = Qh Uh */
        mat *Bt = matrix_new(n, l), *Qh = matrix_new(n, l), *Rh = matrix_new(l, l);
        mat *Uh = matrix_new(l, l), *VhT = matrix_new(l, l);
        gemm_tn(M, Q, Bt);
        qr_econ(Bt, Qh, Rh);
        svd_small(Rh, Uh, *S, VhT);
        gemm_nt(Q, VhT, *U);
        gemm_nn(Qh, Uh, *V);
        matrix_delete(Bt); matrix_delete(Qh); matrix_delete(Rh);
        matrix_delete(Uh); matrix_delete(VhT);
        replace(U, cols(*U, 0, k));
        replace(V, cols(*V, 0, k));
        replace(S, block(*S, 0, k, 0, k));
    } else {
        /* RRA:176-224 : B = Q^T M ; eig(B B^T) ascending ; S = sqrt(evals) ; U = Q Uh ; V = B^T Uh S^-1 */
        mat *B = matrix_new(l, n), *BBt = matrix_new(l, l), *Uh = matrix_new(l, l);
        mat *Sinv = matrix_new(l, l), *UhSinv = matrix_new(l, l);
        double *ev = (double *)calloc((size_t)l, sizeof(double));
        gemm_tn(Q, M, B);
        gemm_nt(B, B, BBt);
        for (int j = 0; j < l; j++)
            for (int i = 0; i <= j; i++) AT(Uh, i, j) = AT(BBt, i, j);
        scipy_LAPACKE_dsyev(COLMAJ, 'V', 'U', l, Uh->d, l, ev);
        for (int i = 0; i < l; i++) AT(*S, i, i) = sqrt(ev[i]);
        gemm_nn(Q, Uh, *U);
        for (int i = 0; i < l; i++) AT(Sinv, i, i) = 1.0 / AT(*S, i, i);
        gemm_nn(Uh, Sinv, UhSinv);
        gemm_tn(B, UhSinv, *V);
        free(ev);
        matrix_delete(B); matrix_delete(BBt); matrix_delete(Uh);
        matrix_delete(Sinv); matrix_delete(UhSinv);
        replace(U, cols(*U, l - k, k));
        replace(V, cols(*V, l - k, k));
        replace(S, block(*S, l - k, k, l - k, k));
    }
}

/* ===================== fixed-rank rSVD (RRA:73-234) ===================== */
void low_rank_svd_rand_decomp_fixed_rank(mat *M, int k, int p, int vnum, int q, int s,
                                         int *frank, mat **U, mat **S, mat **V)
{
    (void)frank; /* never written by the reference (RRA:73-234) */
    int m = M->nrows, n = M->ncols, l = k + p;
    mat *Om = matrix_new(n, l);
    initialize_random_matrix(Om);
    mat *Y = matrix_new(m, l), *Z = matrix_new(n, l);
    mat *Yo = matrix_new(m, l), *Zo = matrix_new(n, l);
    gemm_nn(M, Om, Y);
    /* RRA:101-126: q-1 rounds of (M M^T), orthonormalising when (2j-2)%s / (2j-1)%s == 0 */
    for (int j = 1; j < q; j++) {
        if ((2 * j - 2) % s == 0) { orth_q(Y, Yo); gemm_tn(M, Yo, Z); }
        else gemm_tn(M, Y, Z);
        if ((2 * j - 1) % s == 0) { orth_q(Z, Zo); gemm_nn(M, Zo, Y); }
        else gemm_nn(M, Z, Y);
    }
    mat *Q = matrix_new(m, l);
    orth_q(Y, Q);
    svd_from_q(M, Q, k, vnum, U, S, V);
    matrix_delete(Om); matrix_delete(Y); matrix_delete(Z);
    matrix_delete(Yo); matrix_delete(Zo); matrix_delete(Q);
}

/* ===================== blocked randQB (RRA:1576-1801; randQB_pb RRA:1425-1570) =====================
 * every_step = 0: randQB_pb_new (kstep rule, TOL mode when nstep <= 0, re-orthogonalisation on even
 * steps); every_step = 1: randQB_pb (fixed rank, no kstep rule, re-orthogonalisation on every step
 * after the first, RRA:1500). */
static void qb_blocked_port(mat *M, int kstep, int nstep, double TOL, int q, int s, int *frank,
                            mat **Q, mat **B, int every_step)
{
    int m = M->nrows, n = M->ncols;
    if (!every_step && kstep > (int)(MIN(m, n) / 2)) kstep = (int)MIN(m, n) / 10;   /* RRA:1589-1592 */
    int tol_mode = !every_step && (nstep <= 0);
    if (tol_mode) nstep = (int)(MIN(m, n) / kstep);                    /* RRA:1595-1602 */
    int l = kstep * nstep;
    mat *Om = matrix_new(n, l);
    initialize_random_matrix(Om);
    mat *A = dup(M);
    *Q = matrix_new(m, l);
    *B = matrix_new(l, n);
    mat *Yp = matrix_new(m, kstep), *Qp = matrix_new(m, kstep), *Bp = matrix_new(kstep, n);
    mat *QpBp = matrix_new(m, n), *AtQp = matrix_new(n, kstep), *AtQp2 = matrix_new(n, kstep);
    mat *QptA = matrix_new(kstep, n);
    for (int step = 0; step < nstep; step++) {
        mat *Omp = cols(Om, step * kstep, kstep);
        gemm_nn(A, Omp, Yp);
        matrix_delete(Omp);
        /* RRA:1652-1686: q power rounds */
        for (int j = 1; j <= q; j++) {
            if ((2 * j - 2) % s == 0) {
                orth_q(Yp, Qp);
                if (every_step) {
                    gemm_tn(A, Qp, AtQp);                                  /* RRA:1475 */
                } else {
                    gemm_tn(Qp, A, QptA);
                    mat *t = transpose(QptA);
                    memcpy(AtQp->d, t->d, nel(t) * sizeof(double));
                    matrix_delete(t);
                }
            } else {
                gemm_tn(A, Yp, AtQp);
            }
            if ((2 * j - 1) % s == 0) { orth_q(AtQp, AtQp2); gemm_nn(A, AtQp2, Yp); }
            else gemm_nn(A, AtQp, Yp);
        }
        orth_q(Yp, Qp);
        /* RRA:1703-1732: re-orthogonalise against earlier blocks on even steps only
         * (randQB_pb: every step, RRA:1500-1524) */
        if (step > 0 && (every_step || step % 2 == 0)) {
            int c = step * kstep;
            mat *Qj = cols(*Q, 0, c), *QjtQp = matrix_new(c, kstep), *QjQjtQp = matrix_new(m, kstep);
            gemm_tn(Qj, Qp, QjtQp);
            gemm_nn(Qj, QjtQp, QjQjtQp);
            for (size_t i = 0; i < nel(Yp); i++) Yp->d[i] = Qp->d[i] - QjQjtQp->d[i];
            orth_q(Yp, Qp);
            matrix_delete(Qj); matrix_delete(QjtQp); matrix_delete(QjQjtQp);
        }
        /* RRA:1741-1761: Bp = Qp^T A ; A -= Qp Bp ; Q(:,blk) = Qp ; B(blk,:) = Bp */
        gemm_tn(Qp, A, Bp);
        gemm_nn(Qp, Bp, QpBp);
        for (size_t i = 0; i < nel(A); i++) A->d[i] -= QpBp->d[i];
        memcpy((*Q)->d + (size_t)step * kstep * m, Qp->d, nel(Qp) * sizeof(double));
        for (int j = 0; j < n; j++)
            for (int i = 0; i < kstep; i++) AT(*B, step * kstep + i, j) = AT(Bp, i, j);
        *frank = (step + 1) * kstep;
        if (tol_mode && frob(A) < TOL) break;                          /* RRA:1770-1778 */
    }
    if (tol_mode) {
        replace(Q, cols(*Q, 0, *frank));
        replace(B, rows(*B, 0, *frank));
    }
    matrix_delete(A); matrix_delete(Om); matrix_delete(Yp); matrix_delete(Qp);
    matrix_delete(Bp); matrix_delete(QpBp); matrix_delete(AtQp); matrix_delete(AtQp2);
    matrix_delete(QptA);
}

void randQB_pb_new(mat *M, int kstep, int nstep, double TOL, int q, int s, int *frank,
                   mat **Q, mat **B)
{
    qb_blocked_port(M, kstep, nstep, TOL, q, s, frank, Q, B, 0);
}

void randQB_pb(mat *M, int kstep, int nstep, int q, int s, mat **Q, mat **B)
{
    int frank = 0;
    qb_blocked_port(M, kstep, nstep, 0.0, q, s, &frank, Q, B, 1);
}

/* ===================== blocked rSVD (RRA:239-381) ===================== */
void low_rank_svd_blockrand_decomp_fixed_rank_or_prec(mat *M, int k, int p, double TOL,
                                                      int vnum, int kstep, int q, int s,
                                                      int *frank, mat **U, mat **S, mat **V)
{
    int m = M->nrows, n = M->ncols;
    int rank_mode = (k > 0);
    if (p < kstep && (p + kstep) < MIN(m, n)) p = kstep;              /* RRA:260-262 */
    int nstep = (k + p) / kstep;                                       /* RRA:263: integer division */
    mat *Q, *B;
    randQB_pb_new(M, kstep, nstep, TOL, q, s, frank, &Q, &B);
    if (rank_mode) *frank = k;
    else *frank = (int)round((double)(*frank / (*frank + p + 1e-6)) * (*frank)); /* RRA:278 */
    svd_from_q(M, Q, *frank, vnum, U, S, V);
    matrix_delete(Q);
    matrix_delete(B);
}

/* ===================== pivoted QR (RRA:924-976) ===================== */
void pivotedQR_mkl(mat *M, mat **Q, mat **R, vec **I)
{
    int m = M->nrows, n = M->ncols, k = MIN(m, n);
    int qr_ = (m <= n) ? k : m, qc = k, rr = k, rc = (m <= n) ? n : k;
    mat *W = dup(M);
    int *jpvt = (int *)calloc((size_t)n, sizeof(int));
    double *tau = (double *)calloc((size_t)k, sizeof(double));
    scipy_LAPACKE_dgeqp3(COLMAJ, m, n, W->d, m, jpvt, tau);
    *R = matrix_new(rr, rc);
    for (int j = 0; j < rc; j++)
        for (int i = 0; i < rr && i <= j; i++) AT(*R, i, j) = AT(W, i, j);
    scipy_LAPACKE_dorgqr(COLMAJ, qr_, qc, k, W->d, m, tau);
    *Q = matrix_new(qr_, qc);
    for (int j = 0; j < qc; j++)
        for (int i = 0; i < qr_; i++) AT(*Q, i, j) = AT(W, i, j);
    *I = vector_new(n);
    for (int i = 0; i < n; i++) (*I)->d[i] = (double)(jpvt[i] - 1);
    matrix_delete(W);
    free(jpvt);
    free(tau);
}

/* ===================== deterministic partial pivoted QR (RRA:1159-1334) =====================
 * exact_zero = 0: pivoted_QR_of_specified_rank_or_prec, a pivot column whose squared norm is
 * below 1e-10 ends it (RRA:1250); exact_zero = 1: the rank-only pivoted_QR_of_specified_rank
 * (RRA:1012-1157), which stops only on an exactly zero one (RRA:1069) and has no TOL mode. */
static void pivqr_partial_port(mat *M, int k, double TOL, int *frank, mat **Qk, mat **Rk, vec **I,
                               int exact_zero)
{
    int m = M->nrows, n = M->ncols;
    int tol_mode = !exact_zero && (k <= 0);
    if (tol_mode) k = MIN(m, n);
    mat *Qf = matrix_new(m, m), *R = dup(M), *H = matrix_new(m, 1);
    mat *QHHt = matrix_new(m, m), *HtR = matrix_new(1, n), *HHtR = matrix_new(m, n);
    mat *QH = matrix_new(m, 1);
    for (int i = 0; i < m; i++) AT(Qf, i, i) = 1.0;
    double *nrm = (double *)calloc((size_t)n, sizeof(double));  /* squared column norms */
    for (int j = 0; j < n; j++) {
        double a = 0.0;
        for (int i = 0; i < m; i++) a += AT(M, i, j) * AT(M, i, j);
        nrm[j] = a;
    }
    *frank = 0;
    *I = vector_new(n);
    for (int j = 0; j < n; j++) (*I)->d[j] = j;
    double r22 = 0.0;
    for (int i = 0; i < k; i++) {
        int piv = i;
        double best = nrm[i];
        for (int j = i + 1; j < n; j++)
            if (nrm[j] > best) { best = nrm[j]; piv = j; }
        if (i % 5 == 0) {                                               /* RRA:1225-1258 */
            r22 = 0.0;
            if (tol_mode) {
                for (int j = i; j < n; j++) r22 += nrm[j];
                r22 = sqrt(r22) / n;
            }
        }
        if ((exact_zero ? nrm[piv] == 0.0 : fabs(nrm[piv]) < 1e-10) && i > 0) break;
        if (tol_mode && r22 < TOL) break;
        *frank = i + 1;
        double t = (*I)->d[i]; (*I)->d[i] = (*I)->d[piv]; (*I)->d[piv] = t;
        for (int r = 0; r < m; r++) { t = AT(R, r, i); AT(R, r, i) = AT(R, r, piv); AT(R, r, piv) = t; }
        t = nrm[piv]; nrm[piv] = nrm[i]; nrm[i] = t;
        /* Householder vector scaled so that H H^T is the reflector (RRA:982-1004) */
        memset(H->d, 0, (size_t)m * sizeof(double));
        double nx = 0.0;
        for (int r = i; r < m; r++) { H->d[r] = AT(R, r, i); nx += AT(R, r, i) * AT(R, r, i); }
        H->d[i] -= sqrt(nx);
        double hn = frob(H);
        if (hn > 0) { double sc = sqrt(2.0 / (hn * hn)); for (int r = 0; r < m; r++) H->d[r] *= sc; }
        gemm_tn(H, R, HtR);
        gemm_nn(H, HtR, HHtR);
        for (size_t e = 0; e < nel(R); e++) R->d[e] -= HHtR->d[e];
        gemm_nn(Qf, H, QH);
        gemm_nt(QH, H, QHHt);
        for (size_t e = 0; e < nel(Qf); e++) Qf->d[e] -= QHHt->d[e];
        if (i != n - 1)
            for (int j = i + 1; j < n; j++) nrm[j] -= AT(R, i, j) * AT(R, i, j);
    }
    *Qk = cols(Qf, 0, *frank);
    *Rk = rows(R, 0, *frank);
    matrix_delete(Qf); matrix_delete(R); matrix_delete(H); matrix_delete(QHHt);
    matrix_delete(HtR); matrix_delete(HHtR); matrix_delete(QH);
    free(nrm);
}

void pivoted_QR_of_specified_rank_or_prec(mat *M, int k, double TOL, int *frank,
                                          mat **Qk, mat **Rk, vec **I)
{
    pivqr_partial_port(M, k, TOL, frank, Qk, Rk, I, 0);
}

void pivoted_QR_of_specified_rank(mat *M, int k, int *frank, mat **Qk, mat **Rk, vec **I)
{
    pivqr_partial_port(M, k, 0.0, frank, Qk, Rk, I, 1);
}

/* T = triu(Rk(:,1:r))^{-1} Rk(:,r+1:end) (RRA:1838-1850 and repeats) */
static mat *interp_coeffs(const mat *Rk, int r)
{
    mat *R1 = block(Rk, 0, r, 0, r);
    mat *R2 = block(Rk, 0, r, r, Rk->ncols - r);
    for (int j = 0; j < r; j++)
        for (int i = j + 1; i < r; i++) AT(R1, i, j) = 0.0;
    mat *T = matrix_new(R2->nrows, R2->ncols);
    tri_solve(R1, R2, T);
    matrix_delete(R1);
    matrix_delete(R2);
    return T;
}

/* ===================== IDs (RRA:1807-2111) ===================== */
void id_decomp_fixed_rank_or_prec(mat *M, int k, double TOL, int *frank, vec **I, mat **T)
{
    mat *Qk, *Rk;
    if (k < MIN(M->nrows, M->ncols)) {
        pivoted_QR_of_specified_rank_or_prec(M, k, TOL, frank, &Qk, &Rk, I);
    } else {
        *frank = k;
        pivotedQR_mkl(M, &Qk, &Rk, I);
    }
    *T = interp_coeffs(Rk, *frank);
    matrix_delete(Qk);
    matrix_delete(Rk);
}

void id_rand_decomp_fixed_rank(mat *M, int k, int p, int q, int s, vec **I, mat **T)
{
    int m = M->nrows, n = M->ncols, l = k + p;
    mat *Om = matrix_new(l, m);
    initialize_random_matrix(Om);
    mat *Y = matrix_new(l, n);
    gemm_nn(Om, M, Y);
    /* RRA:1882-1929: q rounds, Z = qr(Y^T,0)^T between the products when scheduled */
    for (int j = 1; j <= q; j++) {
        mat *Z;
        if ((2 * j - 2) % s == 0) {
            mat *Yt = transpose(Y), *Yto = matrix_new(n, l);
            orth_q(Yt, Yto);
            Z = transpose(Yto);
            matrix_delete(Yt); matrix_delete(Yto);
        } else {
            Z = dup(Y);
        }
        replace(&Y, matrix_new(l, m));
        gemm_nt(Z, M, Y);
        matrix_delete(Z);
        if ((2 * j - 1) % s == 0) {
            mat *Yt = transpose(Y), *Yto = matrix_new(m, l);
            orth_q(Yt, Yto);
            Z = transpose(Yto);
            matrix_delete(Yt); matrix_delete(Yto);
        } else {
            Z = dup(Y);
        }
        replace(&Y, matrix_new(l, n));
        gemm_nn(Z, M, Y);
        matrix_delete(Z);
    }
    mat *Qd, *Rd;
    pivotedQR_mkl(Y, &Qd, &Rd, I);
    mat *Rk = rows(Rd, 0, k);
    *T = interp_coeffs(Rk, k);
    matrix_delete(Y); matrix_delete(Qd); matrix_delete(Rd); matrix_delete(Rk);
}

void id_blockrand_decomp_fixed_rank_or_prec(mat *M, int k, int p, double TOL, int kstep,
                                            int q, int s, int *frank, vec **I, mat **T)
{
    int nstep = (k + p) / kstep;                                       /* RRA:1973 */
    int rank_mode = (k > 0);
    if (!rank_mode) nstep = 0;
    mat *Q, *B, *Qk, *Rk;
    randQB_pb_new(M, kstep, nstep, TOL, q, s, frank, &Q, &B);
    pivotedQR_mkl(B, &Qk, &Rk, I);
    if (rank_mode) *frank = k;
    else *frank = (int)round((double)(*frank / (*frank + p + 1e-6)) * (*frank));
    *T = interp_coeffs(Rk, *frank);
    matrix_delete(Q); matrix_delete(B); matrix_delete(Qk); matrix_delete(Rk);
}

/* ===================== decompositions from a given QB (oneapi_code variant) ===================== */
/* oneapi_code/rank_revealing_algorithms_one_api.c:244-300: BBt = B B^T; [Uhat, St, ~] = svd(BBt)
   (descending); S = sqrt(diag(St)) for all l = Q->ncols columns; U = Q Uhat; V = B^T Uhat S^-1. */
void low_rank_svd_rand_decomp_fromQB(mat *Q, mat *B, mat **U, mat **S, mat **V)
{
    int m = Q->nrows, n = B->ncols, l = Q->ncols;
    mat *BBt = matrix_new(l, l), *Uhat = matrix_new(l, l), *St = matrix_new(l, l), *Vt = matrix_new(l, l);
    gemm_nt(B, B, BBt);
    svd_small(BBt, Uhat, St, Vt);
    *U = matrix_new(m, l);
    *S = matrix_new(l, l);
    *V = matrix_new(n, l);
    for (int i = 0; i < l; i++) AT(*S, i, i) = sqrt(AT(St, i, i));
    gemm_nn(Q, Uhat, *U);
    mat *US = matrix_new(l, l);                     /* Uhat S^-1 (1/0 -> inf as in the reference) */
    for (int j = 0; j < l; j++)
        for (int i = 0; i < l; i++) AT(US, i, j) = AT(Uhat, i, j) / AT(*S, j, j);
    gemm_tn(B, US, *V);
    matrix_delete(BBt); matrix_delete(Uhat); matrix_delete(St); matrix_delete(Vt); matrix_delete(US);
}

/* oneapi_code/rank_revealing_algorithms_one_api.c:421-447: k = Q->ncols; [~, Rk, I] = pivotedQR(B);
   T = triu(Rk(:, 1:k))^-1 Rk(:, k+1:n). */
void id_rand_decomp_fromQB(mat *Q, mat *B, vec **I, mat **T)
{
    int k = Q->ncols;
    mat *Qk, *Rk;
    pivotedQR_mkl(B, &Qk, &Rk, I);
    *T = interp_coeffs(Rk, k);
    matrix_delete(Qk); matrix_delete(Rk);
}

/* MIt = M(:,Icol(1:r))^T, then a full-rank deterministic row ID of it (RRA:2042-2051) */
static void row_id_of_selected_columns(mat *M, vec *Icol, int r, vec **Irow, mat **S)
{
    mat *MIt = matrix_new(r, M->nrows);
    for (int c = 0; c < r; c++) {
        int j = (int)Icol->d[c];
        for (int i = 0; i < M->nrows; i++) AT(MIt, c, i) = AT(M, i, j);
    }
    int fr;
    id_decomp_fixed_rank_or_prec(MIt, r, 0, &fr, Irow, S);
    matrix_delete(MIt);
}

void id_two_sided_decomp_fixed_rank_or_prec(mat *M, int k, double TOL, int *frank,
                                            vec **Icol, vec **Irow, mat **T, mat **S)
{
    id_decomp_fixed_rank_or_prec(M, k, TOL, frank, Icol, T);
    row_id_of_selected_columns(M, *Icol, *frank, Irow, S);
}

void id_two_sided_rand_decomp_fixed_rank(mat *M, int k, int p, int q, int s,
                                         vec **Icol, vec **Irow, mat **T, mat **S)
{
    id_rand_decomp_fixed_rank(M, k, p, q, s, Icol, T);
    row_id_of_selected_columns(M, *Icol, k, Irow, S);
}

void id_two_sided_blockrand_decomp_fixed_rank_or_prec(mat *M, int k, int p, double TOL,
                                                      int kstep, int q, int s, int *frank,
                                                      vec **Icol, vec **Irow, mat **T, mat **S)
{
    id_blockrand_decomp_fixed_rank_or_prec(M, k, p, TOL, kstep, q, s, frank, Icol, T);
    row_id_of_selected_columns(M, *Icol, *frank, Irow, S);
}

/* ===================== CUR (RRA:2115-2332) ===================== */
/* V = [I_k; T^T](Icolinv,:), C = M(:,Icol(1:k)), R = M(Irow(1:k),:), U = ((R R^T) \ (R V))^T */
static void cur_from_two_sided(mat *M, int k, vec *Icol, vec *Irow, mat *T,
                               mat **C, mat **U, mat **R)
{
    int m = M->nrows, n = M->ncols;
    mat *V = matrix_new(n, k);
    /* row i of V is row Icolinv[i] of [I;T^T], where Icolinv[Icol[j]] = j (MVF:1195-1201) */
    int *inv = (int *)malloc((size_t)n * sizeof(int));
    for (int j = 0; j < n; j++) inv[(int)Icol->d[j]] = j;
    for (int i = 0; i < n; i++) {
        int r = inv[i];
        for (int c = 0; c < k; c++)
            AT(V, i, c) = (r < k) ? (r == c ? 1.0 : 0.0) : AT(T, c, r - k);
    }
    free(inv);
    *R = matrix_new(k, n);
    for (int j = 0; j < n; j++)
        for (int i = 0; i < k; i++) AT(*R, i, j) = AT(M, (int)Irow->d[i], j);
    *C = matrix_new(m, k);
    for (int c = 0; c < k; c++)
        memcpy((*C)->d + (size_t)c * m, M->d + (size_t)((int)Icol->d[c]) * m, (size_t)m * sizeof(double));
    mat *RRt = matrix_new(k, k), *RV = matrix_new(k, k);
    gemm_nt(*R, *R, RRt);
    gemm_nn(*R, V, RV);
    int *ipiv = (int *)malloc((size_t)k * sizeof(int));
    scipy_LAPACKE_dgesv(COLMAJ, k, k, RRt->d, k, ipiv, RV->d, k);
    *U = transpose(RV);
    free(ipiv);
    matrix_delete(RRt); matrix_delete(RV); matrix_delete(V);
}

void cur_decomp_fixed_rank_or_prec(mat *M, int k, double TOL, int *frank,
                                   mat **C, mat **U, mat **R)
{
    vec *Icol, *Irow;
    mat *T, *S;
    id_two_sided_decomp_fixed_rank_or_prec(M, k, TOL, frank, &Icol, &Irow, &T, &S);
    if (k <= 0) k = *frank;
    cur_from_two_sided(M, k, Icol, Irow, T, C, U, R);
    vector_delete(Icol); vector_delete(Irow); matrix_delete(T); matrix_delete(S);
}

void cur_rand_decomp_fixed_rank(mat *M, int k, int p, int q, int s, mat **C, mat **U, mat **R)
{
    vec *Icol, *Irow;
    mat *T, *S;
    id_two_sided_rand_decomp_fixed_rank(M, k, p, q, s, &Icol, &Irow, &T, &S);
    cur_from_two_sided(M, k, Icol, Irow, T, C, U, R);
    vector_delete(Icol); vector_delete(Irow); matrix_delete(T); matrix_delete(S);
}

void cur_blockrand_decomp_fixed_rank_or_prec(mat *M, int k, int p, double TOL, int kstep,
                                             int q, int s, int *frank,
                                             mat **C, mat **U, mat **R)
{
    vec *Icol, *Irow;
    mat *T, *S;
    id_two_sided_blockrand_decomp_fixed_rank_or_prec(M, k, p, TOL, kstep, q, s, frank,
                                                     &Icol, &Irow, &T, &S);
    cur_from_two_sided(M, *frank, Icol, Irow, T, C, U, R);
    vector_delete(Icol); vector_delete(Irow); matrix_delete(T); matrix_delete(S);
}
