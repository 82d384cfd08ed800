/*
 * rsvd_port.h -- the test oracle's C API (test infrastructure only).
 *
 * The port restates, in our own code, the reference's hot-path algorithms
 * (multi_core_mkl_code/rank_revealing_algorithms_intel_mkl.c, "RRA") on top of
 * LAPACK/CBLAS from scipy's bundled OpenBLAS.  It exports the reference's C API
 * with the same names and the same mat/vec ABI
 * (multi_core_mkl_code/matrix_vector_functions_intel_mkl.h:18-27), so the same
 * ctypes binding drives the reference build (oracle/_ref), this port and the GPU
 * engine.  Only tests/, the smoke check and bench.py's CPU-baseline arm use it.
 */
#ifndef RSVD_PORT_H
#define RSVD_PORT_H

typedef struct { int nrows, ncols; double *d; } mat;
typedef struct { int nrows; double *d; } vec;

typedef void (*rsvd_omega_fn)(void *ctx, int call_index, int nrows, int ncols, double *out);

/* Gaussian test-matrix provider (same ABI as the engine's extension). */
void rsvdpack_set_omega_provider(rsvd_omega_fn fn, void *ctx);
void rsvdpack_reset_omega_counter(void);
int  rsvdpack_omega_calls(void);
void rsvdpack_set_num_threads(int n);

mat *matrix_new(int nrows, int ncols);
vec *vector_new(int nrows);
void matrix_delete(mat *M);
void vector_delete(vec *v);
double get_matrix_frobenius_norm(mat *M);
double get_percent_error_between_two_mats(mat *A, mat *B);
void form_svd_product_matrix(mat *U, mat *S, mat *V, mat *P);
void form_cur_product_matrix(mat *C, mat *U, mat *R, mat *P);
void initialize_random_matrix(mat *M);

void low_rank_svd_rand_decomp_fixed_rank(mat *M, int k, int p, int vnum, int q, int s,
                                         int *frank, mat **U, mat **S, mat **V);
void low_rank_svd_blockrand_decomp_fixed_rank_or_prec(mat *M, int k, int p, double TOL,
                                                      int vnum, int kstep, int q, int s,
                                                      int *frank, mat **U, mat **S, mat **V);
void randQB_pb_new(mat *M, int kstep, int nstep, double TOL, int q, int s, int *frank,
                   mat **Q, mat **B);
void randQB_pb(mat *M, int kstep, int nstep, int q, int s, mat **Q, mat **B);
void pivotedQR_mkl(mat *M, mat **Q, mat **R, vec **I);
void pivoted_QR_of_specified_rank(mat *M, int k, int *frank, mat **Qk, mat **Rk, vec **I);
void pivoted_QR_of_specified_rank_or_prec(mat *M, int k, double TOL, int *frank,
                                          mat **Qk, mat **Rk, vec **I);
void id_decomp_fixed_rank_or_prec(mat *M, int k, double TOL, int *frank, vec **I, mat **T);
void id_rand_decomp_fixed_rank(mat *M, int k, int p, int q, int s, vec **I, mat **T);
void low_rank_svd_rand_decomp_fromQB(mat *Q, mat *B, mat **U, mat **S, mat **V);
void id_rand_decomp_fromQB(mat *Q, mat *B, vec **I, mat **T);
void id_blockrand_decomp_fixed_rank_or_prec(mat *M, int k, int p, double TOL, int kstep,
                                            int q, int s, int *frank, vec **I, mat **T);
void id_two_sided_decomp_fixed_rank_or_prec(mat *M, int k, double TOL, int *frank,
                                            vec **Icol, vec **Irow, mat **T, mat **S);
void id_two_sided_rand_decomp_fixed_rank(mat *M, int k, int p, int q, int s,
                                         vec **Icol, vec **Irow, mat **T, mat **S);
void id_two_sided_blockrand_decomp_fixed_rank_or_prec(mat *M, int k, int p, double TOL,
                                                      int kstep, int q, int s, int *frank,
                                                      vec **Icol, vec **Irow, mat **T, mat **S);
void cur_decomp_fixed_rank_or_prec(mat *M, int k, double TOL, int *frank,
                                   mat **C, mat **U, mat **R);
void cur_rand_decomp_fixed_rank(mat *M, int k, int p, int q, int s, mat **C, mat **U, mat **R);
void cur_blockrand_decomp_fixed_rank_or_prec(mat *M, int k, int p, double TOL, int kstep,
                                             int q, int s, int *frank,
                                             mat **C, mat **U, mat **R);

#endif
