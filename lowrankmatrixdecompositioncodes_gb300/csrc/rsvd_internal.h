// rsvd_internal.h -- internal C++ interfaces of librsvdpack (not installed).
//
// Layering:
//   api.cpp        extern "C" reference API: host mat/vec in, host mat/vec out
//   engine.cu      device-resident algorithms on DM<T> views (rsvd, QB, ID, CUR)
//   k_*.cu         kernels + their launchers declared below
// All device matrices are column-major views {ptr, rows, cols, ld}.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "rsvdpack.h"

namespace rsvd {

using i64 = long long;

// ----------------------------------------------------------------- errors
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};
[[noreturn]] void throw_cuda(cudaError_t e, const char *what, const char *file, int line);
[[noreturn]] void fail(int code, const std::string &msg);
void set_error(int code, const std::string &msg);   // thread-local last error

#define RSVD_CK(x)                                                              \
    do {                                                                        \
        cudaError_t e_ = (x);                                                   \
        if (e_ != cudaSuccess) ::rsvd::throw_cuda(e_, #x, __FILE__, __LINE__);  \
    } while (0)
#define RSVD_LAUNCH_CK() RSVD_CK(cudaGetLastError())

// ----------------------------------------------------------------- device views
template <typename T>
struct DM {
    T *p = nullptr;
    i64 r = 0, c = 0, ld = 0;
    __host__ __device__ T *col(i64 j) const { return p + j * ld; }
    __host__ __device__ T &at(i64 i, i64 j) const { return p[i + j * ld]; }
    DM sub(i64 r0, i64 c0, i64 nr, i64 nc) const { return DM{p + r0 + c0 * ld, nr, nc, ld}; }
    DM cols(i64 c0, i64 nc) const { return sub(0, c0, r, nc); }
};

// Stream-ordered device buffer (cudaMallocAsync on the calling thread's stream).
class DBuf {
  public:
    DBuf() = default;
    DBuf(size_t bytes, cudaStream_t s);
    ~DBuf();
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    DBuf(DBuf &&o) noexcept : p_(o.p_), n_(o.n_), s_(o.s_) { o.p_ = nullptr; o.n_ = 0; }
    DBuf &operator=(DBuf &&o) noexcept;
    void *get() const { return p_; }
    size_t bytes() const { return n_; }

  private:
    void *p_ = nullptr;
    size_t n_ = 0;
    cudaStream_t s_ = nullptr;
};

// Leading dimension used for device copies: rows rounded up to 32 elements so that
// every column starts on a 128-byte boundary (TMA needs 16-byte strides).
inline i64 pad_ld(i64 rows) { return ((rows + 31) / 32) * 32; }

template <typename T>
struct DMat {  // owning device matrix
    DBuf buf;
    DM<T> v;
    DMat() = default;
    DMat(i64 r, i64 c, cudaStream_t s, bool zero = true);
    operator DM<T>() const { return v; }
};

// ----------------------------------------------------------------- per-thread context
struct Ctx {
    cudaStream_t stream = nullptr;
    int device = -1;
    int sms = 0;
    int cc_major = 0, cc_minor = 0;
    int *d_flags = nullptr;       // device status words (see k_common.cuh: FLAG_*)
    rsvdpack_opts opts{};
    rsvdpack_timing timing{};
    long long launches = 0;
    // TF32 mode: products A X (A the MN-major operand, which kind::tf32 cannot read) take A
    // as a two-part BF16 split (hi + lo, 16 mantissa bits) instead of one BF16 copy (7 bits).
    // Set by the fixed-precision block loop, whose sketches must resolve the deflated matrix.
    bool ax_split = false;
    // Cholesky breakdown checks deferred to the end of a solve (FP32-data fixed-rank solves):
    // the factorisations leave FLAG_CHOL_BREAKDOWN set instead of returning to the host after
    // each one; if it is set at the end, the solve is repeated with chol_force_hh (Householder QR
    // for every orthonormalisation).
    bool chol_deferred = false;
    bool chol_force_hh = false;
    // kernels may read pageable host memory directly (cudaDevAttrPageableMemoryAccess: GB300
    // with a Grace host, over NVLink-C2C)
    bool pageable_access = false;
    // device-time phase marks of the current call (PhaseTimer), resolved by phase_collect()
    struct PhaseMark {
        cudaEvent_t a, b;
        double *acc;
    };
    std::vector<PhaseMark> marks;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
};
Ctx &ctx();                       // initialises the device on first use; throws RSVD_ERR_NO_DEVICE

// Device time of a region on the engine stream, added to *acc (a rsvdpack_timing field) when
// the call ends: two pooled events per region, no synchronisation inside the region.
struct PhaseTimer {
    cudaEvent_t b = nullptr;
    double *acc;
    explicit PhaseTimer(double *acc_ms);
    ~PhaseTimer();
};
void phase_reset();                // start of a call
void phase_collect();              // end of a call: waits for the stream, resolves the marks
const rsvdpack_opts &global_opts();

// The learned proposal's network (host copy; null when none is installed).
struct ProposalModel {
    std::vector<float> params, norm, margin;
};
const ProposalModel *proposal_model();
void set_proposal_model(ProposalModel m);
void check_device_flags(Ctx &c);  // throws if a kernel reported a timeout / breakdown

// Gaussian test-matrix provider (host side).
bool omega_provider_active();
unsigned long long &philox_calls();   // per-thread Philox stream counter (reset with the provider counter)
void omega_fill_host(int nrows, int ncols, double *out);  // serves the next request

// ----------------------------------------------------------------- kernel launchers (k_dense.cu)
// C = alpha * op(A) * op(B) + beta * C  (CUDA cores; double or float)
template <typename T>
void gemm_simt(cudaStream_t s, bool ta, bool tb, i64 M, i64 N, i64 K, T alpha, const T *A,
               i64 lda, const T *B, i64 ldb, T beta, T *C, i64 ldc);
template <typename T>
void gemm(cudaStream_t s, bool ta, bool tb, T alpha, DM<T> A, DM<T> B, T beta, DM<T> C);

template <typename Ts, typename Td>
void convert(cudaStream_t s, DM<Ts> src, DM<Td> dst);      // dst = (Td)src, same shape
// dst = (float)src and dst2 = bf16(dst), one pass (C-API upload with the BF16 copy of A)
template <typename Ts>
void convert_f32_bf16(cudaStream_t s, DM<Ts> src, DM<float> dst, DM<__nv_bfloat16> dst2);
// hi = bf16(x) (round to nearest), lo = bf16(x - hi): x = hi + lo to ~2^-16 relative.
void split_bf16(cudaStream_t s, DM<float> src, DM<__nv_bfloat16> hi, DM<__nv_bfloat16> lo);
template <typename T>
void fill_zero(cudaStream_t s, DM<T> a);
template <typename T>
void set_identity(cudaStream_t s, DM<T> a);
template <typename T>
void transpose(cudaStream_t s, DM<T> src, DM<T> dst);      // dst (c x r) = src^T
template <typename T>
void gather_cols(cudaStream_t s, DM<T> src, const int *idx, DM<T> dst);  // dst(:,j)=src(:,idx[j])
template <typename T>
void gather_rows(cudaStream_t s, DM<T> src, const int *idx, DM<T> dst);  // dst(i,:)=src(idx[i],:)
template <typename T>
void sub_inplace(cudaStream_t s, DM<T> a, DM<T> b);        // a -= b
template <typename T>
double frob_norm(cudaStream_t s, DM<T> a);                  // synchronous
void philox_gaussian(cudaStream_t s, unsigned long long seed, unsigned long long offset, DM<double> out);
void philox_gaussian(cudaStream_t s, unsigned long long seed, unsigned long long offset, DM<float> out);

// Small dense FP64 kernels.
// Upper Cholesky G = R^T R in place (upper triangle); lower triangle zeroed.
// Returns false on breakdown (pivot <= rel_tol * original diagonal).  Synchronous.
bool cholesky_upper(cudaStream_t s, DM<double> G, double rel_tol, int *d_flag);
// Q = Y * R^-1 for upper-triangular R (FP64), row by row.
template <typename T>
void trsm_right_upper(cudaStream_t s, DM<T> Y, DM<double> R, DM<T> Q);
// X = triu(R)^-1 * B  (left, upper, FP64), one column of B per warp.
void trsm_left_upper(cudaStream_t s, DM<double> R, DM<double> B, DM<double> X);
// One-sided Jacobi SVD of square G (n x n, FP64): G = U diag(sv) V^T, sorted descending.
// G is overwritten.  U, V: n x n.  Returns the sweep count.
int jacobi_svd(cudaStream_t s, DM<double> G, DM<double> U, DM<double> V, double *d_sv, int *d_flag);
// Default precision mode of the reference API of this library (defined by its api.cu build).
int api_default_precision();

// Householder QR of a tall matrix: Q (r x c) explicit, R (c x c) upper.  FP64/FP32 tall data.
template <typename T>
void householder_qr(cudaStream_t s, DM<T> Y, DM<T> Q, DM<double> R);

// ----------------------------------------------------------------- pivoted QR (k_pivqr.cu)
// Column-pivoted Householder QR with LAPACK dgeqp3 pivoting (all columns free):
// on exit A holds R in its upper triangle and the reflectors below it, tau[min(m,n)],
// jpvt[n] holds 0-based source columns.
void pivqr_lapack(cudaStream_t s, DM<double> A, double *d_tau, int *d_jpvt);
// Form Q (m x qc) from the reflectors stored in A (dorgqr).
void form_q_from_reflectors(cudaStream_t s, DM<double> A, const double *d_tau, int nrefl, DM<double> Q);
// The reference's own partial pivoted QR (rank_revealing_algorithms_intel_mkl.c:1159-1334).
// Returns frank; fills Q (m x m workspace) and R (m x n) in place.  zero_tol: a pivot column
// whose squared norm is below it ends the factorisation (1e-10, RRA:1250); 0 means exactly zero
// (the rank-only pivoted_QR_of_specified_rank, RRA:1069).
int pivqr_rsvdpack(cudaStream_t s, DM<double> R, DM<double> Q, int k, double TOL, bool tol_mode,
                   int *d_jpvt, double zero_tol = 1e-10);
// Solve A X = B in place (B <- X) by LU with partial pivoting (dgesv); false if singular.
bool lu_solve(cudaStream_t s, DM<double> A, DM<double> B, int *d_flag);
// G = Y^T Y (c x c, FP64) for tall Y: FP64 products for double data; for float data,
// FP32 products summed in FP32 over 256-row chunks and in FP64 across chunks.
template <typename T>
void gram(cudaStream_t s, DM<T> Y, DM<double> G);

}  // namespace rsvd

namespace rsvd {
// ----------------------------------------------------------------- tensor-core GEMM (k_gemm_tc.cu)
// kind 0: tf32 operands (fp32 in memory), kind 1: bf16 operands.
// D (M x N, fp32, column-major, ldd) = alpha * sum_k Aop(i,k) X(k,j), where
//   a_mn == true : Aop(i,k) = A[i + k*lda]   (A column-major M x K: the "A X" form)
//   a_mn == false: Aop(i,k) = A[k + i*lda]   (A column-major K x M: the "A^T X" form)
//   X(k,j) = X[k + j*ldx]                    (X column-major K x N)
// epi 0: D = alpha*acc (split-K allowed: splits_hint 0 = auto, 1 = none, >1 = forced);
// epi 1: D = C - alpha*acc, with per-CTA sums of squares of D written to fro_part
//        (gridDim.x * gridDim.y doubles) when fro_part is not null.
// Requirements: A, X 16-byte aligned; lda*esize and ldx*esize multiples of 16 bytes.
void tc_gemm(cudaStream_t s, int kind, bool a_mn, const void *A, long long lda, const void *X, long long ldx,
             int M, int N, int K, float alpha, float *D, long long ldd, int epi, const float *C, long long ldc,
             double *fro_part, int splits_hint);
// The same product with K split into up to 3 segments that accumulate into one result:
// acc = sum_s Aop_s^T-contracted X_s (each segment its own operands, leading dimensions and
// K; all share M, N and a_mn), in segment order.  Used for the three terms of a 3xTF32
// product (small terms first), so that they make one pass over the output.
struct TcSeg {
    const void *A;
    long long lda;
    const void *X;
    long long ldx;
    int K;
};
// Optional extra outputs of an update (epi 1): the new D split as TF32 hi / lo (hi = D
// rounded to TF32, lo = D - hi) and as BF16 hi / lo -- the operands the next 3xTF32 and
// two-part BF16 products read -- written by the epilogue (or by separate passes when the
// update cannot use the TMA epilogue).
struct TcSplitOut {
    float *hi, *lo;
    long long ld;
    __nv_bfloat16 *bhi, *blo;
    long long ldb;
};
void tc_gemm_segs(cudaStream_t s, int kind, bool a_mn, int nseg, const TcSeg *seg, int M, int N, float alpha,
                  float *D, long long ldd, int epi, const float *C, long long ldc, double *fro_part, int splits_hint,
                  const TcSplitOut *so = nullptr);
// 3xTF32 (FP32-accurate) products on the tf32 pipe: split_tf32 writes hi = tf32(X) and
// lo = X - hi; tc_gemm_3xtf32 computes D = A^T X (A K-major, K x M) from split operands.
void split_tf32(cudaStream_t s, const float *X, long long ldx, long long r, long long c, float *hi, float *lo,
                long long ldo);
void tc_gemm_3xtf32(cudaStream_t s, const float *Ahi, const float *Alo, long long lda, const float *Xhi,
                    const float *Xlo, long long ldx, int M, int N, int K, float *D, long long ldd);
// C (M x N) -= A^T X (3xTF32, one pass over C, in place); fro_part as for tc_gemm's update.
void tc_update_3xtf32(cudaStream_t s, const float *Ahi, const float *Alo, long long lda, const float *Xhi,
                      const float *Xlo, long long ldx, int M, int N, int K, float *Cm, long long ldc,
                      double *fro_part, const TcSplitOut *so = nullptr);
// ----------------------------------------------------------------- tiled triangular steps (k_chol.cu)
// G (n x n, FP64, upper triangle read) -> R, G = R^T R (upper, zero below), compute type S.
// dinv (optional): receives the inverses of R's 32 x 32 diagonal tiles (ceil(n/32) row-major
// tiles), which tri_inv_tiles consumes.  false on breakdown (pivot <= rel_tol * G_jj).
template <typename S>
bool chol_factor(cudaStream_t s, DM<double> G, double rel_tol, int *d_flag, S *dinv);
template <typename S, typename To>
void tri_inv_tiles(cudaStream_t s, DM<double> R, const S *dinv, DM<To> X);   // X = R^-1
template <typename S>
void tri_mul_upper(cudaStream_t s, DM<double> A, DM<double> B, DM<double> C);   // C = A B (upper)
// Q = Y R^-1 (R from chol_factor, dinv its inverted diagonal tiles), order <= 288;
// false when the order is too large (nothing queued).
template <typename T>
bool trsm_right_tiles(cudaStream_t s, DM<T> Y, DM<double> R, const T *dinv, DM<T> Q);
// The FP32 CholeskyQR pass on packed upper 32 x 32 tiles (orders <= 288): the Gram is
// reduced straight into FP32 tiles (Gt: ceil(n/32)(ceil(n/32)+1)/2 tiles of 1024 floats),
// factored in one CTA (Gt then holds R; Rout optional FP64 copy), and applied by the slab
// triangular solve.
void gram_tiles_f32(cudaStream_t s, DM<float> Y, float *Gt, DM<double> *G);
bool chol_tiles_f32(cudaStream_t s, float *Gt, int n, double rel_tol, int *d_flag, float *dinv, DM<double> *Rout);
// Binary matrix files (k_io.cu): the header (two integers of hdr_bytes each) and the streaming
// load of the row-major entries (real_bytes each) into a column-major device matrix of dtype.
bool binary_file_shape(const char *fname, int hdr_bytes, long long *m, long long *n);
void load_binary_to_device(const char *fname, int hdr_bytes, int real_bytes, int dtype, void *dA, long long lda,
                           long long *m_out, long long *n_out);
// C = A B (FP32, column-major) in 3xTF32 on the tensor cores (FP32-accurate products).
void gemm_nn_3xtf32(cudaStream_t s, DM<float> A, DM<float> B, DM<float> C);
void trsm_right_tiles_f32(cudaStream_t s, DM<float> Y, int n, const float *Rt, const float *dinv, DM<float> Q);
// Both in one cooperative launch (the solve of block column J overlaps the factorisation of
// block J + 1): -1 when not possible here (the caller runs the two above), 1, or 0 on breakdown.
int chol_trsm_fused_f32(cudaStream_t s, float *Gt, int n, double rel_tol, float *dinv, DM<double> *Rout, DM<float> Y,
                        DM<float> Q);
}  // namespace rsvd

namespace rsvd {
// ----------------------------------------------------------------- learned proposal MLP (k_mlp.cu)
int mlp_param_count();
void mlp_dims(int *d);                                      // 4 layer widths
void mlp_forward(cudaStream_t s, const float *P, const float *norm, const float *X, int B, float *Y);
void mlp_train_step(cudaStream_t s, float *P, float *M, float *V, const float *norm, const float *X, const float *T,
                    const float *reached, int B, float lr, int step, float *loss, float *G);
}  // namespace rsvd

namespace rsvd {
// ----------------------------------------------------------------- small l x l steps (k_small.cu)
// Compute type S: double in the FP64 mode, float in the mixed modes (storage is FP64).
template <typename S>
bool cholesky_small(cudaStream_t s, DM<double> G, double rel_tol, int *d_flag);
template <typename S>
// Returns the sweep count when want_sweeps (a host read of the count, i.e. a stream sync), else 0.
int jacobi_small(cudaStream_t s, DM<double> G, DM<double> U, DM<double> V, double *d_sv, int *d_flag,
                 bool want_sweeps = true);
}  // namespace rsvd

namespace rsvd {
// ----------------------------------------------------------------- FP64-accurate products on the FP32 pipe (k_df64.cu)
// x = (hi + lo) * 2^(exp - 1023): an FP64 matrix split once into two FP32 parts, scaled on the
// device by a power of two so that the largest |x| lies in [1, 2).
struct Df64Split {
    DBuf buf;
    float *hi = nullptr, *lo = nullptr;
    int *exp = nullptr;          // device scalar: biased exponent field of the largest |x| (0: no scale)
    i64 r = 0, c = 0, ld = 0;
    // exp_src (device, optional): the biased exponent field to scale by (e.g. 1023: no scaling,
    // for matrices with entries of order one), instead of the largest |x| found by a pass over x
    Df64Split(cudaStream_t s, DM<double> x, const int *exp_src = nullptr);
    struct Df64View view() const;
};
// A split operand as the product kernel reads it (hi, lo: FP32 column-major, ld; exp: device scale).
struct Df64View {
    const float *hi = nullptr, *lo = nullptr;
    i64 r = 0, c = 0, ld = 0;
    const int *exp = nullptr;
    Df64View rows(i64 r0, i64 nr) const { return Df64View{hi + r0, lo + r0, nr, c, ld, exp}; }
};
inline Df64View Df64Split::view() const { return Df64View{hi, lo, r, c, ld, exp}; }
// Optional second output of a product: the result split as hi = fl32(C), lo = fl32(C - hi) (no scale).
struct Df64Out {
    float *hi, *lo;
    i64 ld;
};
// C = alpha op(A) op(B) + beta C with double-float accumulation (~2^-47 relative per product term).
void df64_gemm(cudaStream_t s, bool ta, bool tb, double alpha, const Df64Split &A, const Df64Split &B, double beta,
               DM<double> C);
void df64_gemm(cudaStream_t s, bool ta, bool tb, double alpha, Df64View A, Df64View B, double beta, DM<double> C,
               const Df64Out *out);
// C0 = A0^T A0 and C1 = A1^T A1 (same shapes) in one launch, upper-triangle tiles only: entries
// (i, j) with i <= j are exact to the product's accuracy; tiles below the diagonal are not written.
void df64_gram_pair(cudaStream_t s, Df64View A0, DM<double> C0, Df64View A1, DM<double> C1);
// ----------------------------------------------------------------- SVD refinement (k_small.cu)
// X (n x n, FP64) and approximate right singular vectors V (n x n, columns; FP32-accurate, e.g.
// from the FP32 Jacobi) -> the SVD of X to FP64 accuracy: U, V (n x n) and sv (device, n values),
// descending.  V is overwritten; U may not alias V.  `steps` first-order corrections.
// Refinement steps after the FP32 Jacobi: the first takes FP32-accurate vectors to ~1e-12, the
// second to the FP64 floor, the last settles nearly equal pairs coupled beyond 2e-5.  Three steps
// leave the singular values as accurate but the vectors of clustered values orthogonal only to
// ~5e-10; the fourth brings them to ~1e-12.
constexpr int REFINE_STEPS = 4;
void svd_refine(cudaStream_t s, DM<double> X, DM<double> V, DM<double> U, double *d_sv, int steps);
// The mixed-precision l x l SVD: FP32 one-sided Jacobi, then svd_refine (FP64-accurate result).
void small_svd_refined(cudaStream_t s, DM<double> G, DM<double> U, DM<double> V, double *d_sv, int *d_flag);
}  // namespace rsvd
