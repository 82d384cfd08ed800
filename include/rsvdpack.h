/*
 * rsvdpack.h -- public C ABI of librsvdpack.so, the GB300 (sm_103a) engine for
 * RSVDPACK's randomized low-rank decompositions.
 *
 * Part 1 reproduces the reference's C API as a drop-in: the same struct layouts,
 * function names, argument meanings, output shapes and ownership rules.
 *   - mat / vec and their helpers: multi_core_mkl_code/matrix_vector_functions_intel_mkl.h
 *   - decompositions:             multi_core_mkl_code/rank_revealing_algorithms_intel_mkl.h
 * Matrices are column-major on the host (ld = nrows; double, or float in librsvdpack_f32.so).  Inputs are
 * borrowed and never modified; outputs are allocated by the callee with
 * matrix_new / vector_new (calloc) and freed by the caller with
 * matrix_delete / vector_delete.  Index vectors hold 0-based integers as rsvd_real values.
 * All calls are synchronous: device work is finished when they return.
 * Calls are re-entrant per host thread (each thread owns a CUDA stream).
 *
 * The reference returns void and ignores LAPACK's info; so does this drop-in.
 * Failures (bad arguments, CUDA errors, device timeouts) never exit(): the
 * outputs are set to NULL and rsvdpack_last_error() reports a non-zero code.
 *
 * Part 2 holds additive extensions (precision modes, sketch-matrix provider,
 * device-resident entry points, batched and learned paths, per-call timing).  They have
 * no counterpart in the reference unless stated.
 */
#ifndef RSVDPACK_H
#define RSVDPACK_H

#include <stddef.h>
#include <stdint.h>
#include <sys/time.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ============================== Part 1: reference API ============================== */

/* Index and element types of Part 1, one library per variant of the reference, all three built
 * from the same sources over the same engine:
 *   librsvdpack.so      int dimensions, double data: multi_core_mkl_code (the default);
 *   librsvdpack64.so    int64_t dimensions, double data (RSVDPACK_INDEX64):
 *                       multi_core_mkl_code_64bit/matrix_vector_functions_intel_mkl.h:20-28 and every
 *                       dimension, rank and step argument of its rank_revealing_algorithms_intel_mkl.h,
 *                       for matrices of more than 2^31 entries;
 *   librsvdpack_f32.so  int64_t dimensions, float data and float TOL (RSVDPACK_REAL32):
 *                       oneapi_code/matrix_vector_functions_one_api.h:19-32 and
 *                       rank_revealing_algorithms_one_api.h; its default precision mode is
 *                       RSVD_PREC_FP32 (the oneAPI variant computes in single precision).
 * Define RSVDPACK_INDEX64 or RSVDPACK_REAL32 before including this header to compile against the
 * matching library.  Part 2 is the same in all three (int sizes, typed device pointers). */
#if defined(RSVDPACK_REAL32)
typedef int64_t rsvd_int;
typedef float rsvd_real;
#elif defined(RSVDPACK_INDEX64)
typedef int64_t rsvd_int;
typedef double rsvd_real;
#else
typedef int rsvd_int;
typedef double rsvd_real;
#endif

/* matrix_vector_functions_intel_mkl.h:18-27 (rsvd_int dimensions, rsvd_real data, column-major) */
typedef struct {
    rsvd_int nrows, ncols;
    rsvd_real *d;
} mat;

typedef struct {
    rsvd_int nrows;
    rsvd_real *d;
} vec;

/* ---- storage and element access: matrix_vector_functions_intel_mkl.h:31-58 ---- */
mat *matrix_new(rsvd_int nrows, rsvd_int ncols);
vec *vector_new(rsvd_int nrows);
void matrix_delete(mat *M);
void vector_delete(vec *v);
void matrix_set_element(mat *M, rsvd_int row_num, rsvd_int col_num, rsvd_real val);
rsvd_real matrix_get_element(mat *M, rsvd_int row_num, rsvd_int col_num);
void vector_set_element(vec *v, rsvd_int row_num, rsvd_real val);
rsvd_real vector_get_element(vec *v, rsvd_int row_num);

/* ---- binary matrix files: matrix_vector_functions_intel_mkl.h:60-64 (format: m and n as
 *      rsvd_int -- int32 in librsvdpack.so, int64 in librsvdpack64.so and librsvdpack_f32.so as in
 *      multi_core_mkl_code_64bit/matrix_vector_functions_intel_mkl.c:86-87 and
 *      oneapi_code/matrix_vector_functions_one_api.c:79-80 -- then m*n rsvd_real values in
 *      row-major order; matrix_vector_functions_intel_mkl.c:77-133) ---- */
mat *matrix_load_from_binary_file(char *fname);
void matrix_write_to_binary_file(mat *M, char *fname);

/* ---- helpers callers use around the decompositions ---- */
void matrix_copy(mat *D, mat *S);                                 /* :92-94 */
void matrix_build_transpose(mat *Mt, mat *M);                     /* :100-101 */
rsvd_real get_matrix_frobenius_norm(mat *M);                      /* :116-117 */
rsvd_real get_percent_error_between_two_mats(mat *A, mat *B);     /* :288-289 */
rsvd_real vector_get2norm(vec *v);                                /* :83 */
void initialize_diagonal_matrix(mat *D, vec *data);               /* :199: D(i,i) = data(i) */
void initialize_identity_matrix(mat *D);                          /* :204 (diagonal bounded by min(m, n)) */
void matrix_get_col(mat *M, rsvd_int j, vec *column_vec);          /* :158 */
void matrix_set_col(mat *M, rsvd_int j, vec *column_vec);          /* :161 */

/* ---- the other host-side mat / vec helpers of matrix_vector_functions_intel_mkl.h (same
 *      meanings; entries outside either object are never touched; vector_get_min_element /
 *      vector_get_max_element compare the values truncated to rsvd_int, as the reference does) ---- */
void matrix_print(mat *M);
void vector_print(vec *v);
void vector_set_data(vec *v, rsvd_real *data);
void vector_scale(vec *v, rsvd_real scalar);
void matrix_scale(mat *M, rsvd_real scalar);
void vector_copy(vec *d, vec *s);
void matrix_hard_threshold(mat *M, rsvd_real TOL);
void vector_sub(vec *a, vec *b);
void matrix_sub(mat *A, mat *B);
void matrix_sub_column_times_row_vector(mat *A, vec *u, vec *v);
void vector_get_min_element(vec *v, rsvd_int *minindex, rsvd_real *minval);
void vector_get_max_element(vec *v, rsvd_int *maxindex, rsvd_real *maxval);
rsvd_real vector_dot_product(vec *u, vec *v);
rsvd_real get_matrix_max_abs_element(mat *M);
rsvd_real get_matrix_column_norm_squared(mat *M, rsvd_int colnum);
rsvd_real matrix_getmaxcolnorm(mat *M);
void compute_matrix_column_norms(mat *M, vec *column_norms);
void invert_diagonal_matrix(mat *Dinv, mat *D);
void project_vector(vec *v, vec *u, vec *p);
void build_orthonormal_basis_from_mat(mat *A, mat *Q);
void matrix_get_row(mat *M, rsvd_int i, vec *row_vec);
void matrix_set_row(mat *M, rsvd_int i, vec *row_vec);
void matrix_get_selected_columns(mat *M, rsvd_int *inds, mat *Mc);
void matrix_set_selected_columns(mat *M, rsvd_int *inds, mat *Mc);
void matrix_get_selected_rows(mat *M, rsvd_int *inds, mat *Mr);
void matrix_set_selected_rows(mat *M, rsvd_int *inds, mat *Mr);
void matrix_copy_symmetric(mat *S, mat *M);
void matrix_keep_only_upper_triangular(mat *M);
void fill_vector_from_row_list(vec *input, vec *inds, vec *output);
void matrix_copy_first_rows(mat *M_out, mat *M);
void matrix_copy_first_columns(mat *M_out, mat *M);
void matrix_copy_first_columns_with_param(mat *D, mat *S, rsvd_int num_columns);
void matrix_copy_first_k_rows_and_columns(mat *M_out, mat *M);
void matrix_copy_all_rows_and_last_columns_from_indexk(mat *M_out, mat *M, rsvd_int k);
void fill_matrix_from_first_rows(mat *M, rsvd_int k, mat *M_k);
void fill_matrix_from_last_rows(mat *M, rsvd_int k, mat *M_k);
void fill_matrix_from_first_columns(mat *M, rsvd_int k, mat *M_k);
void fill_matrix_from_last_columns(mat *M, rsvd_int k, mat *M_k);
void fill_matrix_from_last_columns_from_specified_one(mat *M, rsvd_int k, mat *M_k);
void fill_matrix_from_lower_right_corner(mat *M, rsvd_int k, mat *M_out);
void fill_matrix_from_first_columns_from_list(mat *M, vec *I, rsvd_int k, mat *M_k);
void fill_matrix_from_first_rows_from_list(mat *M, vec *I, rsvd_int k, mat *M_k);
void fill_matrix_from_last_columns_from_list(mat *M, vec *I, rsvd_int k, mat *M_k);
void resize_matrix_by_columns(mat **M, rsvd_int k);
void resize_matrix_by_columns_from_end(mat **M, rsvd_int k);
void resize_matrix_by_rows(mat **M, rsvd_int k);
void resize_matrix_by_rows_from_end(mat **M, rsvd_int k);
void append_matrices_horizontally(mat *A, mat *B, mat *C);
void append_matrices_vertically(mat *A, mat *B, mat *C);
void vector_build_rewrapped(vec *Iinv, vec *I);
void initialize_random_matrix(mat *M);                            /* :128-129 */
void matrix_matrix_mult(mat *A, mat *B, mat *C);                  /* :132-133 */
void matrix_transpose_matrix_mult(mat *A, mat *B, mat *C);        /* :136-137 */
void matrix_matrix_transpose_mult(mat *A, mat *B, mat *C);        /* :140-141 */
void matrix_vector_mult(mat *M, vec *x, vec *y);                  /* :149: y = M x */
void matrix_transpose_vector_mult(mat *M, vec *x, vec *y);        /* :153: y = M^T x */
/* :213 in place inverse of an upper-triangular matrix (the strictly lower part is left as it is) */
void invert_upper_triangular_matrix(mat *Minv);
/* :354 A X = B for upper-triangular A of order B->nrows; solve_type 2 inverts A in place first, as
 * the reference does; the other types give the triangular solve */
void upper_triangular_system_solve(mat *A, mat *B, mat *X, rsvd_int solve_type);
/* :328 eigenvalues ascending into evals and eigenvectors into the columns of S (the upper triangle
 * of S defines the symmetric matrix, as for LAPACK dsyev 'V' 'U') */
void compute_evals_and_evecs_of_symm_matrix(mat *S, vec *evals);
/* :357 A X = B by LU with partial pivoting; X and B receive the solution, A is left as it is */
void square_matrix_system_solve(mat *A, mat *X, mat *B);
/* :333, :338 Householder QR with LAPACK's reflector signs (dgeqrf + dorgqr), m >= n: M = Q R with
 * Q (m x n, caller-allocated) and, for compact_QR_factorization, R (n x n, caller-allocated; its
 * upper triangle is written, as the reference writes it). */
void compact_QR_factorization(mat *M, mat *Q, mat *R);
void QR_factorization_getQ(mat *M, mat *Q);
void form_svd_product_matrix(mat *U, mat *S, mat *V, mat *P);     /* :343-344 */
void form_cur_product_matrix(mat *C, mat *U, mat *R, mat *P);     /* :346-347 */
#if defined(RSVDPACK_REAL32)
rsvd_real get_seconds_frac(rsvd_real start, rsvd_real end);  /* one_api.h:367: end - start (omp_get_wtime values) */
#else
double get_seconds_frac(struct timeval start_timeval, struct timeval end_timeval); /* :359-360 */
#endif

/* ---- decompositions: rank_revealing_algorithms_intel_mkl.h ---- */
/* :5  fixed-rank randomized SVD.  q means q-1 rounds of (M M^T); vnum 1 (or >2): QR of
 *     B^T route, singular values descending; vnum 2: eig(B B^T) route, ascending.
 *     U m x k, S k x k dense diagonal, V n x k.  frank is not written (as in the reference). */
void low_rank_svd_rand_decomp_fixed_rank(mat *M, rsvd_int k, rsvd_int p, rsvd_int vnum, rsvd_int q, rsvd_int s,
                                         rsvd_int *frank, mat **U, mat **S, mat **V);
/* :7  blocked randomized SVD (rank k, or absolute Frobenius tolerance TOL when k <= 0) */
void low_rank_svd_blockrand_decomp_fixed_rank_or_prec(mat *M, rsvd_int k, rsvd_int p, rsvd_real TOL,
                                                      rsvd_int vnum, rsvd_int kstep, rsvd_int q, rsvd_int s,
                                                      rsvd_int *frank, mat **U, mat **S, mat **V);
/* :67 blocked randomized QB (nstep <= 0 selects the TOL mode) */
void randQB_pb_new(mat *M, rsvd_int kstep, rsvd_int nstep, rsvd_real TOL, rsvd_int q, rsvd_int s, rsvd_int *frank,
                   mat **Q, mat **B);
/* oneapi_code/rank_revealing_algorithms_one_api.h:13-14: randQB_pb2 is randQB_pb_new (the same
 * algorithm, one_api.c:605-815); :57 randQB_pb: nstep blocks of kstep, q power rounds, every block
 * after the first re-orthogonalised against the earlier ones (rank_revealing_algorithms_intel_mkl.c
 * :1425-1570), Q m x (kstep nstep), B (kstep nstep) x n. */
void randQB_pb2(mat *M, rsvd_int kstep, rsvd_int nstep, rsvd_real TOL, rsvd_int q, rsvd_int s, rsvd_int *frank,
                mat **Q, mat **B);
void randQB_pb(mat *M, rsvd_int kstep, rsvd_int nstep, rsvd_int q, rsvd_int s, mat **Q, mat **B);
/* :43 full column-pivoted QR, M(:,I) = Q R (LAPACK dgeqp3 pivoting, all columns free) */
void pivotedQR_mkl(mat *M, mat **Q, mat **R, vec **I);
/* :45 Householder vector of x(ind1:ind2) into column 0 of H, scaled so that I - H H^T reflects it */
void get_householder_matrix(vec *x, rsvd_int ind1, rsvd_int ind2, mat *H);
/* :52 partial pivoted Householder QR of rank k, or of precision TOL when k <= 0 */
void pivoted_QR_of_specified_rank_or_prec(mat *M, rsvd_int k, rsvd_real TOL, rsvd_int *frank,
                                          mat **Qk, mat **Rk, vec **I);
/* :47 partial pivoted Householder QR of rank k >= 1 (rank_revealing_algorithms_intel_mkl.c
 *     :1012-1157): the rank-or-precision routine's rank mode, except that only an exactly vanished
 *     pivot column ends it early (RRA:1069; the other stops below 1e-10, RRA:1250) */
void pivoted_QR_of_specified_rank(mat *M, rsvd_int k, rsvd_int *frank, mat **Qk, mat **Rk, vec **I);
/* :73 column ID, T = Rk1^-1 Rk2 */
void id_decomp_fixed_rank_or_prec(mat *M, rsvd_int k, rsvd_real TOL, rsvd_int *frank, vec **I, mat **T);
/* :76 randomized column ID (row sketch (k+p) x n, q power rounds) */
void id_rand_decomp_fixed_rank(mat *M, rsvd_int k, rsvd_int p, rsvd_int q, rsvd_int s, vec **I, mat **T);
/* decompositions from a given QB (Q m x l, B l x n; the QB split of the oneAPI variant,
 * oneapi_code/rank_revealing_algorithms_one_api.h:6,10, with this header's rsvd_int dimensions):
 * low_rank_svd_rand_decomp_fromQB: U (m x l), S (l x l, descending), V (n x l) from the SVD of
 * B B^T, V = B^T Uhat S^-1; id_rand_decomp_fromQB: column ID of B with k = Q->ncols,
 * I (0-based pivots of B, as doubles) and T = R11^-1 R12 (k x (n - k)).  FP64. */
void low_rank_svd_rand_decomp_fromQB(mat *Q, mat *B, mat **U, mat **S, mat **V);
void id_rand_decomp_fromQB(mat *Q, mat *B, vec **I, mat **T);
/* :79 blocked randomized column ID */
void id_blockrand_decomp_fixed_rank_or_prec(mat *M, rsvd_int k, rsvd_int p, rsvd_real TOL, rsvd_int kstep,
                                            rsvd_int q, rsvd_int s, rsvd_int *frank, vec **I, mat **T);
/* :84 two-sided ID */
void id_two_sided_decomp_fixed_rank_or_prec(mat *M, rsvd_int k, rsvd_real TOL, rsvd_int *frank,
                                            vec **Icol, vec **Irow, mat **T, mat **S);
/* :87 randomized two-sided ID.  The reference header names the parameters (k,l,p,s);
 *     the definition (rank_revealing_algorithms_intel_mkl.c:2060) uses (k,p,q,s). */
void id_two_sided_rand_decomp_fixed_rank(mat *M, rsvd_int k, rsvd_int p, rsvd_int q, rsvd_int s,
                                         vec **Icol, vec **Irow, mat **T, mat **S);
/* :90 blocked randomized two-sided ID */
void id_two_sided_blockrand_decomp_fixed_rank_or_prec(mat *M, rsvd_int k, rsvd_int p, rsvd_real TOL,
                                                      rsvd_int kstep, rsvd_int q, rsvd_int s, rsvd_int *frank,
                                                      vec **Icol, vec **Irow, mat **T, mat **S);
/* :95 CUR */
void cur_decomp_fixed_rank_or_prec(mat *M, rsvd_int k, rsvd_real TOL, rsvd_int *frank,
                                   mat **C, mat **U, mat **R);
/* :98 randomized CUR */
void cur_rand_decomp_fixed_rank(mat *M, rsvd_int k, rsvd_int p, rsvd_int q, rsvd_int s, mat **C, mat **U, mat **R);
/* :101 blocked randomized CUR */
void cur_blockrand_decomp_fixed_rank_or_prec(mat *M, rsvd_int k, rsvd_int p, rsvd_real TOL, rsvd_int kstep,
                                             rsvd_int q, rsvd_int s, rsvd_int *frank,
                                             mat **C, mat **U, mat **R);
/* :12-25 the older randomized SVD entry points, each one of the routines above with fixed parameters
 * (rank_revealing_algorithms_intel_mkl.c:385-700): svd1 = low_rank_svd_rand_decomp_fixed_rank with
 * p = 0, vnum = 2, q = 1; svd2 = p = 0, vnum = 1, q = 1; svd3 = p = 0, vnum = 1 with q, s; svd4 =
 * randQB_pb(kstep, nstep, p, s = 1) followed by eig(B B^T), pairs ascending.  (The header names
 * svd4's last argument s; the definition uses it as p.) */
void randomized_low_rank_svd1(mat *M, rsvd_int k, mat **U, mat **S, mat **V);
void randomized_low_rank_svd2(mat *M, rsvd_int k, mat **U, mat **S, mat **V);
void randomized_low_rank_svd3(mat *M, rsvd_int k, rsvd_int q, rsvd_int s, mat **U, mat **S, mat **V);
void randomized_low_rank_svd4(mat *M, rsvd_int kstep, rsvd_int nstep, rsvd_int p, mat **U, mat **S, mat **V);
/* :105-120 approximation reports (print norms and percent error, as the reference does).
 * use_pivoted_QR_decomp_for_approximation frees Qk and Rk, as the reference does. */
void use_low_rank_svd_for_approximation(mat *M, mat *U, mat *S, mat *V);
void use_pivoted_QR_decomp_for_approximation(mat *M, mat *Qk, mat *Rk, vec *I);
void use_QB_decomp_for_approximation(mat *M, mat *Q, mat *B);
void use_id_decomp_for_approximation(mat *M, mat *T, vec *I, rsvd_int k);
void use_id_two_sided_decomp_for_approximation(mat *M, mat *T, mat *S, vec *Icol, vec *Irow, rsvd_int k);
void use_cur_decomp_for_approximation(mat *M, mat *C, mat *U, mat *R);

/* ============================== Part 2: extensions ============================== */

/* Status codes reported by rsvdpack_last_error() (per host thread). */
enum {
    RSVD_OK = 0,
    RSVD_ERR_ARGUMENT = 1,     /* invalid sizes / parameters */
    RSVD_ERR_CUDA = 2,         /* CUDA runtime error */
    RSVD_ERR_NO_DEVICE = 3,    /* no usable sm_103a device */
    RSVD_ERR_NUMERIC = 4,      /* non-finite input or breakdown that the fallbacks could not repair */
    RSVD_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up */
    RSVD_ERR_ALLOC = 6         /* device or host allocation failed */
};
int rsvdpack_last_error(void);
const char *rsvdpack_last_error_string(void);
void rsvdpack_clear_error(void);

/* Arithmetic of the large products (sketch, power rounds, projections) and of the
 * storage of A on the device.  Small k x k work: in RSVD_PREC_FP64, FP64 Cholesky and triangular
 * solves; in every mode the l x l SVD of the randomized SVD routines is the FP32 one-sided Jacobi
 * refined to FP64 accuracy by double-float products (singular values to ~1e-14 relative of the
 * l x l factor; absolute ~1e-14 sigma_1 for strongly graded factors), and the Cholesky
 * factorisations of FP32-data Grams run in FP32.  Pivot decisions are FP64 in every mode. */
enum {
    RSVD_PREC_FP64 = 0,   /* FP64 data and arithmetic: reproduces the reference (default) */
    RSVD_PREC_FP32 = 1,   /* A and tall factors FP32, CUDA-core FP32 products */
    RSVD_PREC_TF32 = 2,   /* A FP32, tcgen05 kind::tf32 products, FP32 accumulate */
    RSVD_PREC_BF16 = 3,   /* A FP32 + BF16 copy, tcgen05 kind::f16 (bf16) sketch products */
    RSVD_PREC_FP64X = 4   /* A FP64; the large products FP64-accurate on the FP32 pipe (double-
                             float accumulation, ~2^-46 relative per term, ~5x GB300's FP64 rate) */
};

typedef struct {
    int precision;            /* RSVD_PREC_* */
    int use_provider;         /* 1: Gaussian test matrices come from the registered provider
                                 when one is set (default 1); 0: always on-device Philox */
    unsigned long long seed;  /* Philox key for on-device test matrices */
    int verbose;              /* print the reference's progress lines (default 0) */
    int learned;              /* randQB_pb_new in TOL mode, FP32 data: let the learned proposal
                                 (rsvdpack_load_proposal_model) pick the sketch width and power
                                 count of one single-shot QB, verified against TOL, with the
                                 plain adaptive loop as the fallback (default 0) */
    int reserved[7];
} rsvdpack_opts;

void rsvdpack_get_opts(rsvdpack_opts *opts);
void rsvdpack_set_opts(const rsvdpack_opts *opts);

/* Gaussian test-matrix provider.  The reference draws every test matrix with
 * initialize_random_matrix (matrix_vector_functions_intel_mkl.c:458-486), time-seeded.
 * A provider makes runs repeatable and lets a caller hand the engine the same test
 * matrices it hands another implementation: request number call_index (0-based,
 * counted since registration or the last reset) fills nrows*ncols doubles in
 * column-major order.  Pass fn = NULL to go back to on-device Philox. */
typedef void (*rsvd_omega_fn)(void *ctx, int call_index, int nrows, int ncols, double *out);
void rsvdpack_set_omega_provider(rsvd_omega_fn fn, void *ctx);
void rsvdpack_reset_omega_counter(void);
int rsvdpack_omega_calls(void);

/* Device and build information: fills name (>= 64 bytes); returns the SM count, or
 * a negative value when no usable device is present. */
int rsvdpack_device_info(char *name, int name_len, int *cc_major, int *cc_minor);

/* ---- device-resident entry points (no counterpart in the reference) ----
 * For callers whose matrices already live in GPU memory.  Pointers are device
 * pointers; matrices are column-major with the given leading dimensions (elements).
 * dtype: RSVD_DT_F64 or RSVD_DT_F32 (FP32 data is computed in the current precision
 * mode's arithmetic; FP64 data always in FP64).  The work is queued on the calling
 * thread's engine stream (rsvdpack_stream()), ordered after all work already queued on the
 * legacy default stream (work on other streams must be complete or ordered by the caller);
 * the call returns after it finishes.
 * Return value: RSVD_OK or an RSVD_ERR_* code (also kept in rsvdpack_last_error()). */
enum { RSVD_DT_F64 = 0, RSVD_DT_F32 = 1, RSVD_DT_BF16 = 2 /* rsvdpack_dev_sketch only */ };

/* Fixed-rank rSVD with the reference's semantics (as low_rank_svd_rand_decomp_fixed_rank).
 * Outputs: U (m x k, ldu), S (k values, double, reference order), V (n x k, ldv), all
 * caller-allocated device buffers, U and V in the input dtype. */
int rsvdpack_dev_svd_fixed_rank(const void *dA, int dtype, long long lda, int m, int n, int k, int p,
                                int vnum, int q, int s, void *dU, long long ldu, double *dS, void *dV,
                                long long ldv);

/* One sketch product with the engine's product kernel for the current precision:
 * trans == 0: Y (m x w) = A X with X (n x w);  trans == 1: Y (n x w) = A^T X with X (m x w).
 * dtype RSVD_DT_BF16: A is a BF16 matrix (16-byte aligned, lda a multiple of 8), X and Y are
 * FP32; X is rounded to BF16 and the product is one tensor-core kernel with FP32 accumulation
 * (the form the mixed-precision solve uses after its once-per-call BF16 copy of A). */
int rsvdpack_dev_sketch(const void *dA, int dtype, long long lda, int m, int n, const void *dX, long long ldx,
                        int w, void *dY, long long ldy, int trans);

/* FP32-accurate tensor-core products (3xTF32): x = hi + lo with hi = x rounded to TF32; the
 * terms lo*hi, hi*lo and hi*hi accumulate on the tf32 pipe in FP32 (long K in chains of ~256,
 * summed with compensation).  FP32 device data, column-major: A is K x M (lda), X is K x N (ldx).
 * rsvdpack_dev_gemm_3xtf32:   D (M x N, ldd) = A^T X.
 * rsvdpack_dev_update_3xtf32: C (M x N, ldc) -= A^T X in place in one pass over C (the
 *   blocked-QB deflation A_res -= Q_j B_j with A = Q_j^T, X = B_j); fro2 (host, optional)
 *   receives ||C||_F^2 of the result.  No counterpart in the reference. */
int rsvdpack_dev_gemm_3xtf32(const float *dA, long long lda, const float *dX, long long ldx, int M, int N, int K,
                             float *dD, long long ldd);
int rsvdpack_dev_update_3xtf32(const float *dA, long long lda, const float *dX, long long ldx, int M, int N, int K,
                               float *dC, long long ldc, double *fro2);

/* Residual norms of a low-rank approximation on device data (the reference reports only the
 * Frobenius error, via get_percent_error_between_two_mats on the formed product): *fro receives
 * ||A - U diag(S) V^T||_F and *spec the spectral norm estimate (block power iteration, `iters`
 * rounds of 8 vectors, then Rayleigh-Ritz: a lower bound that converges to ||.||_2); either may be
 * NULL.  A m x n (lda), U m x k (ldu), V n x k (ldv) in dtype RSVD_DT_F64 or RSVD_DT_F32; S: k
 * doubles on the device.  The residual is formed once on the device (double-float products for
 * FP64 data) and kept in FP32. */
int rsvdpack_dev_residual_norms(const void *dA, int dtype, long long lda, int m, int n, const void *dU,
                                long long ldu, const double *dS, const void *dV, long long ldv, int k, int iters,
                                double *fro, double *spec);

/* The reference's binary matrix files (matrix_load_from_binary_file, matrix_vector_functions_
 * intel_mkl.c:77-133: two header integers m, n of this library's rsvd_int width, then the m x n
 * entries of this library's rsvd_real type row by row) streamed straight into device memory.
 * rsvdpack_binary_file_shape reads the header.  rsvdpack_dev_load_binary reads the file in
 * ~32 MiB chunks of whole rows through two pinned staging buffers, copies each chunk to the
 * device on its own stream and transposes it there into dA (column-major, leading dimension
 * lda >= m, in dtype RSVD_DT_F64, RSVD_DT_F32 or RSVD_DT_BF16, round to nearest), so that file
 * reads, copies and transposes overlap; m and n (optional) receive the shape.  Synchronous: the
 * matrix is complete when the call returns. */
int rsvdpack_binary_file_shape(const char *fname, long long *m, long long *n);
int rsvdpack_dev_load_binary(const char *fname, int dtype, void *dA, long long lda, long long *m, long long *n);

/* FP64-accurate product on the FP32 pipe (no counterpart in the reference):
 * C (M x N, ldc) = alpha op(A) op(B) + beta C, op(X) = X^T when its flag is set; FP64 device
 * data, column-major.  Each operand is split once into FP32 parts (hi + lo, scaled on the device
 * by a power of two) and every product term is accumulated in double-float arithmetic (exact
 * FP32 two-product, compensated two-sum): ~2^-46 relative per term, about five times the rate of
 * GB300's FP64 pipe.  The product time is reported as rsvdpack_last_timing()->sketch_ms. */
int rsvdpack_dev_gemm_df64(int ta, int tb, int M, int N, int K, double alpha, const double *dA, long long lda,
                           const double *dB, long long ldb, double beta, double *dC, long long ldc);

/* The calling thread's engine stream (a cudaStream_t), for event timing by callers. */
void *rsvdpack_stream(void);

/* ---- batched fixed-rank rSVD (no counterpart in the reference, which takes one matrix per
 * call): low_rank_svd_rand_decomp_fixed_rank with vnum = 1 on `count` independent FP32
 * device matrices of uneven size, in one persistent launch captured in a CUDA graph.
 * Matrix i: A_i (m[i] x n[i], lda[i]) -> U_i (m[i] x k[i], ldu[i]), S_i (k[i] doubles,
 * descending), V_i (n[i] x k[i], ldv[i]); the arrays hold device pointers and are copied at
 * plan creation.  Test matrices are Philox Gaussians (stream = seed, item index).
 * Limits: k[i] + p <= min(m[i], n[i]), k[i] + p <= 72, n[i] * (k[i] + p) <= 54,000.
 * Execute returns RSVD_OK, or RSVD_ERR_NUMERIC if some item broke down (its outputs are
 * then left unwritten). */
typedef struct rsvdpack_batch_plan rsvdpack_batch_plan;
rsvdpack_batch_plan *rsvdpack_batch_plan_create(int count, const int *m, const int *n, const int *k, int p, int q,
                                                int s, const float *const *dA, const long long *lda,
                                                float *const *dU, const long long *ldu, double *const *dS,
                                                float *const *dV, const long long *ldv, unsigned long long seed);
int rsvdpack_batch_plan_execute(rsvdpack_batch_plan *plan);
void rsvdpack_batch_plan_destroy(rsvdpack_batch_plan *plan);
/* The configuration a plan runs: lanes per Jacobi pair (4, 8, 16 or 32 = one warp per pair) and
 * the offset (0 or 1) added to the narrowest register-tile column-group count of the per-item
 * products.  Plan creation looks the batch's class -- (max k + p, max n / 64, max m / 64, q) -- up in
 * the autotuner's table (RSVDPACK_TUNE_FILE, else $HOME/.cache/rsvdpack/batch_tune.txt) or, when
 * absent, times the eight candidates on a strided sample of the batch (2 x SMs matrices) and
 * records the fastest; RSVDPACK_NO_TUNE=1 keeps the default (8, 0).  *tuned: 1 measured now, 2 read
 * from the table, 0 default; *tune_ms: the choice's time on the sample. */
int rsvdpack_batch_plan_info(const rsvdpack_batch_plan *plan, int *lanes_per_pair, int *col_group_offset,
                             int *tuned, double *tune_ms);

/* The l x l steps on their own (device FP64 storage, column-major; compute in FP32 when
 * fp32 != 0, else FP64).  rsvdpack_dev_small_svd: G (n x n) = U diag(S) V^T, S descending,
 * by one-sided Jacobi (the engine's l x l SVD); fp32 == 2 selects the refined form the
 * randomized SVD routines use: the FP32 Jacobi followed by four FP64-accurate refinement steps
 * (double-float products on the FP32 pipe, exact FP64 rotations of nearly equal pairs): singular
 * values to ~1e-14 relative, singular vectors orthonormal to ~1e-12 (~1e-10 for singular values
 * closer than ~1e-6 relative), for factors whose singular values span up to ~6 decades (the
 * accuracy is absolute, ~1e-13 sigma_1, so it degrades for values far below sigma_1; fp32 == 0 is
 * the form for strongly graded factors); returns the FP32 or FP64 sweep count or a negative
 * RSVD_ERR_* code.  rsvdpack_dev_small_cholesky: G = R^T R in place (upper R, lower
 * part zeroed); returns RSVD_OK, RSVD_ERR_NUMERIC on breakdown, or another RSVD_ERR_* code. */
int rsvdpack_dev_small_svd(double *dG, int n, long long ldg, double *dU, long long ldu, double *dS, double *dV,
                           long long ldv, int fp32);
int rsvdpack_dev_small_cholesky(double *dG, int n, long long ldg, int fp32);

/* Allocation-free sketch product Y (n x w) = A^T X (A m x n, X m x w; FP32, tcgen05 kind::tf32,
 * split-K).  No counterpart in the reference.  For callers that cannot allocate GPU memory at
 * the point of the call -- code under an external memory manager or a budget that forbids
 * driver allocations, or code that must not take the implicit device synchronisation of
 * cudaMalloc / cudaFree.  It allocates nothing and creates nothing: it uses the caller's buffers,
 * the caller's stream (a cudaStream_t, may be 0), and a 32 MiB scratch array inside the library
 * that each GPU loading the library holds until exit.  Limit: round_up(n, 32) * w <= 4,194,272
 * and m > 32; larger products return RSVD_ERR_ARGUMENT.  The first call on each device (made
 * with that device current) looks up the scratch address; make it before any stream capture.
 * Calls share the scratch: calls that overlap on the GPU race, so serialise them.
 * A, X, Y 16-byte aligned; lda, ldx multiples of 4.  Synchronous (it waits for its stream), so
 * it cannot be captured: on a stream that is capturing it queues nothing and returns
 * RSVD_ERR_ARGUMENT.  Returns RSVD_OK or RSVD_ERR_*. */
int rsvdpack_dev_sketch_t_noalloc(const float *dA, long long lda, int m, int n, const float *dX,
                                  long long ldx, int w, float *dY, long long ldy, void *stream);

/* ---- the learned rank / power-count proposal's network (no counterpart in the reference):
 * an MLP 36 -> 64 -> 64 -> 2 (ReLU) whose inputs are the R-diagonal features of a 32-column
 * probe sketch and whose outputs are log2(width / 32) of the single-shot range finder for
 * q = 1 and q = 2 power iterations.  Parameters: one flat FP32 array (W_l row-major in x out,
 * then b_l, layer by layer); norm = [mean(36), inv_std(36)] of the inputs.  All pointers are
 * device pointers; calls run on the engine stream and return after it finishes. */
int rsvdpack_mlp_info(int *dims /* 4 layer widths */, int *nparams);
/* Fixed-rank or fixed-precision blocked QB on device data (randQB_pb_new semantics; nstep <= 0
 * selects the TOL mode, TOL absolute).  Q (m x frank, ldq) and B (frank x n, ldb) go to
 * caller buffers with room for cap columns / rows; *frank receives the rank.  With
 * rsvdpack_opts.learned set, FP32 data and a proposal model installed, the TOL mode runs the
 * learned proposal (rsvdpack_last_timing()->learned_path reports which path ran). */
int rsvdpack_dev_qb(const void *dA, int dtype, long long lda, int m, int n, int kstep, int nstep, double TOL,
                    int q, int s, void *dQ, long long ldq, void *dB, long long ldb, int cap, int *frank);

/* Install the proposal network used when rsvdpack_opts.learned is set (host arrays, copied):
 * params (nparams floats), norm (2 x input width), margin (one log2 safety margin per output).
 * rsvdpack_load_proposal_model reads the same from a weights file (magic "RSVDMLP1"). */
int rsvdpack_set_proposal_model(const float *params, int nparams, const float *norm, int nnorm,
                                const float *margin, int nmargin);
int rsvdpack_load_proposal_model(const char *path);
int rsvdpack_mlp_forward(const float *dP, const float *dnorm, const float *dX, int batch, float *dY);
/* One training step: forward, loss (squared error; a target whose run did not reach the
 * tolerance, dReached[i] == 0, only penalises predictions below it), backward into dG, and an
 * Adam update of dP (state dM, dV; step >= 1) when lr > 0.  *dloss receives the batch loss. */
int rsvdpack_mlp_train_step(float *dP, float *dM, float *dV, const float *dnorm, const float *dX, const float *dT,
                            const float *dReached, int batch, float lr, int step, float *dloss, float *dG);

/* Per-call phase timing of the last decomposition on this thread (milliseconds). */
typedef struct {
    double upload_ms, sketch_ms, orth_ms, small_ms, download_ms, total_ms;
    long long gemm_launches, kernel_launches;
    int learned_path;   /* last fixed-precision QB: 0 plain loop, 1 learned proposal accepted,
                           2 learned proposal rejected by the residual check (plain loop ran) */
    int pad_;
} rsvdpack_timing;
void rsvdpack_last_timing(rsvdpack_timing *t);

#ifdef __cplusplus
}
#endif

#endif /* RSVDPACK_H */
