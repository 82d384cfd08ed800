// engine.h -- device-resident decompositions (called by api.cu).
//
// Every routine takes A as a device view and leaves its results on the device.  The
// steps follow multi_core_mkl_code/rank_revealing_algorithms_intel_mkl.c ("RRA"); the
// products and orthonormalisations are GPU kernels:
//   Q = orth(Y)  : CholeskyQR2 (FP64 Cholesky of an FP64-accumulated Gram), Householder
//                  QR when Cholesky breaks down.  Same column space as the reference's
//                  dgeqrf+dorgqr Q; columns may differ in sign, which no output depends on
//                  beyond the sign of singular-vector pairs.
//   l x l SVD    : one-sided Jacobi (FP64).
//   pivoting     : k_pivqr.cu (dgeqp3 rule / the reference's own rule).
#pragma once
#include "rsvd_internal.h"

namespace rsvd {

template <typename T>
struct SvdOut {
    DMat<T> U, V;
    std::vector<double> S;   // length k, in the reference's order for vnum
};

template <typename T>
struct QBOut {
    DMat<T> Q, B;
    int frank = 0;
};

struct IdOut {
    std::vector<int> I;      // 0-based permutation (length n)
    DMat<double> T;          // k x (n - k)
    int frank = 0;
};

struct TwoSidedOut {
    std::vector<int> Icol, Irow;
    DMat<double> T, S;
    int frank = 0;
};

struct CurOut {
    DMat<double> C, U, R;
    int frank = 0;
};

struct PivQROut {
    DMat<double> Q, R;
    std::vector<int> I;
    int frank = 0;
};

// Large products (sketch, power rounds, projections): precision-mode dispatch.
template <typename T>
void prod(cudaStream_t s, bool ta, bool tb, T alpha, DM<T> A, DM<T> B, T beta, DM<T> C);
// Drop the per-call BF16 operand copies (called at the end of every API call).
void release_operand_cache();
// The call's cached BF16 copy of X (same shape and leading dimension as to_bf16 would make).
void adopt_bf16_copy(DM<float> X, DMat<__nv_bfloat16> &&copy);
// Large FP64 products (FP64 GEMM, or double-float on the FP32 pipe in the FP64X mode).
void prod_f64(cudaStream_t s, bool ta, bool tb, double alpha, DM<double> A, DM<double> B, double beta, DM<double> C);
bool fp64x_mode();

// Gaussian test matrix (r x c): provider when registered (and enabled), else Philox.
template <typename T>
DMat<T> make_omega(i64 r, i64 c);

template <typename T>
void orth(DM<T> Y, DM<T> Q, DM<double> *R, int passes = 2);

template <typename T>
SvdOut<T> svd_fixed_rank(DM<T> A, int k, int p, int vnum, int q, int s);
template <typename T>
SvdOut<T> svd_blockrand(DM<T> A, int k, int p, double TOL, int vnum, int kstep, int q, int s, int *frank);
// Blocked QB rules: randQB_pb_new / randQB_pb2 (RRA:1576-1801, oneapi_code
// rank_revealing_algorithms_one_api.c:605-815: kstep above min(m,n)/2 shrinks to min(m,n)/10,
// nstep <= 0 selects the TOL mode, re-orthogonalisation on even steps) or randQB_pb (RRA:1425-1570,
// one_api.c:451-600: fixed rank, no kstep rule, re-orthogonalisation on every step after the first).
enum QbRule { QB_PB_NEW = 0, QB_PB = 1 };
template <typename T>
QBOut<T> qb_blocked(DM<T> A, int kstep, int nstep, double TOL, int q, int s, QbRule rule = QB_PB_NEW);

PivQROut pivoted_qr_full(DM<double> A);
PivQROut pivoted_qr_partial(DM<double> A, int k, double TOL, double zero_tol = 1e-10);
IdOut id_det(DM<double> A, int k, double TOL);
IdOut id_rand(DM<double> A, int k, int p, int q, int s);
IdOut id_blockrand(DM<double> A, int k, int p, double TOL, int kstep, int q, int s);
TwoSidedOut id_two_sided(DM<double> A, IdOut col);
SvdOut<double> svd_from_qb(DM<double> Q, DM<double> B);
IdOut id_from_qb(DM<double> B, int k);
CurOut cur_from_two_sided(DM<double> A, int k, const TwoSidedOut &ts);
// ||A - U diag(S) V^T||_F and ||.||_2 (k_resid.cu); S on the device (k values); either output may be
// null; the spectral value is the Rayleigh-Ritz estimate after `iters` block power rounds.
template <typename T>
void residual_norms(DM<T> A, DM<T> U, const double *dS, DM<T> V, double *fro, double *spec, int iters);

}  // namespace rsvd
