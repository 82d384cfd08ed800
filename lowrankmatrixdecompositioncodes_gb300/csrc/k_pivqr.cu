// k_pivqr.cu -- column-pivoted QR on the GPU (FP64), the pivot kernels of the ID / CUR paths.
//
// Two pivoting rules, each reproducing one reference code path:
//  * LAPACK rule (pivotedQR_mkl -> dgeqp3, rank_revealing_algorithms_intel_mkl.c:924-976):
//    pivot = first argmax of the partial column norms vn1; reflector as dlarfg
//    (beta = -sign(alpha)|x|); after each step the partial norms are downdated with
//    LAPACK's rule vn1 *= sqrt(max(0,(1+t)(1-t))), t = |A(i,j)|/vn1, and recomputed
//    from the trailing column when (1-t^2)(vn1/vn2)^2 <= sqrt(eps) (the open-source
//    dlaqp2 / dlaqps recipe).  The pivots equal dgeqp3's whenever the norms are not
//    tied at rounding level.
//  * RSVDPACK rule (pivoted_QR_of_specified_rank_or_prec, rank_revealing_algorithms_intel_mkl.c:1159-1334):
//    pivot = first argmax of squared column norms, downdated by subtraction;
//    reflector h = x - |x| e_i scaled so that I - h h^T reflects; stop on a zero norm
//    or, in TOL mode, when sqrt(sum of remaining squared norms)/n < TOL (tested every
//    5 steps).
// Each step is two launches: a one-block "select" kernel (argmax, swap, reflector) and a
// column-parallel "apply" kernel (reflect the trailing columns, update norms).  A device
// control word carries the pivot and the stop decision between them, so the host never
// waits inside the loop.
#include "rsvd_internal.h"
#include "k_common.cuh"

#include <algorithm>
#include <cmath>

namespace rsvd {

namespace {

struct PivCtl {
    int stop;    // 1 once the factorisation has ended
    int frank;   // steps taken
    int pvt;     // pivot chosen in the current step
    int pad;
    double r22;  // RSVDPACK rule: last tested remainder norm
};

// Block argmax of v[i..n) (first index among equal maxima).  All threads get (val, idx).
__device__ void block_argmax(const double *v, int i, int n, double &bestv, int &besti) {
    __shared__ double sv[32];
    __shared__ int si[32];
    double bv = -1.0;
    int bi = n;
    for (int j = i + threadIdx.x; j < n; j += blockDim.x) {
        const double x = v[j];
        if (x > bv) { bv = x; bi = j; }   // strided scan keeps the first index per thread
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { sv[wid] = bv; si[wid] = bi; }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        bv = (lane < nw) ? sv[lane] : -1.0;
        bi = (lane < nw) ? si[lane] : n;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
        }
        if (lane == 0) { sv[0] = bv; si[0] = bi; }
    }
    __syncthreads();
    bestv = sv[0];
    besti = si[0];
    __syncthreads();
}

__device__ void swap_columns(double *A, i64 ld, i64 m, int a, int b) {
    if (a == b) return;
    for (i64 r = threadIdx.x; r < m; r += blockDim.x) {
        const double t = A[r + a * ld];
        A[r + a * ld] = A[r + b * ld];
        A[r + b * ld] = t;
    }
}

// ------------------------------------------------------------------ LAPACK rule
__global__ void colnorm_kernel(const double *A, i64 ld, i64 m, int n, double *vn1, double *vn2, int *jpvt) {
    const int lane = threadIdx.x & 31;
    for (int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); j < n; j += gridDim.x * (blockDim.x >> 5)) {
        double a = 0.0;
        for (i64 r = lane; r < m; r += 32) a = fma(A[r + j * ld], A[r + j * ld], a);
        a = warp_sum(a);
        if (lane == 0) {
            vn1[j] = sqrt(a);
            vn2[j] = vn1[j];
            jpvt[j] = j;
        }
    }
}

__global__ void __launch_bounds__(1024) lapack_select_kernel(double *A, i64 ld, i64 m, int n, int i, double *vn1,
                                                             double *vn2, int *jpvt, double *tau) {
    __shared__ double sc[32];
    double bv;
    int pvt;
    block_argmax(vn1, i, n, bv, pvt);
    if (pvt >= n) pvt = i;
    if (pvt != i) {
        swap_columns(A, ld, m, pvt, i);
        if (threadIdx.x == 0) {
            const int t = jpvt[pvt]; jpvt[pvt] = jpvt[i]; jpvt[i] = t;
            vn1[pvt] = vn1[i];
            vn2[pvt] = vn2[i];
        }
    }
    __syncthreads();
    // dlarfg on A(i:m, i)
    double sig = 0.0;
    for (i64 r = i + 1 + threadIdx.x; r < m; r += blockDim.x) sig = fma(A[r + i * ld], A[r + i * ld], sig);
    sig = block_sum(sig, sc);
    const double alpha = A[i + i * ld];
    double beta = alpha, t = 0.0, scale = 0.0;
    if (sig != 0.0) {
        const double nrm = sqrt(alpha * alpha + sig);
        beta = (alpha >= 0.0) ? -nrm : nrm;
        t = (beta - alpha) / beta;
        scale = 1.0 / (alpha - beta);
    }
    for (i64 r = i + 1 + threadIdx.x; r < m; r += blockDim.x) A[r + i * ld] *= scale;
    __syncthreads();
    if (threadIdx.x == 0) {
        A[i + i * ld] = beta;
        tau[i] = t;
    }
}

// one warp per trailing column j in (i, n)
__global__ void lapack_apply_kernel(double *A, i64 ld, i64 m, int n, int i, const double *tau, double *vn1,
                                    double *vn2, double tol3z) {
    const int lane = threadIdx.x & 31;
    const int j = i + 1 + (int)((blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5);
    if (j >= n) return;
    const double t = tau[i];
    double *x = A + (i64)j * ld;
    const double *v = A + (i64)i * ld;
    if (t != 0.0) {
        double w = 0.0;
        for (i64 r = i + 1 + lane; r < m; r += 32) w = fma(v[r], x[r], w);
        w = warp_sum(w) + x[i];
        const double f = t * w;
        for (i64 r = i + 1 + lane; r < m; r += 32) x[r] -= f * v[r];
        if (lane == 0) x[i] -= f;
    }
    __syncwarp();
    const double nv = vn1[j];
    if (nv != 0.0) {
        double tt = fabs(x[i]) / nv;
        tt = fmax(0.0, (1.0 + tt) * (1.0 - tt));
        const double ratio = nv / vn2[j];
        const double t2 = tt * ratio * ratio;
        if (t2 <= tol3z) {
            double a = 0.0;
            for (i64 r = i + 1 + lane; r < m; r += 32) a = fma(x[r], x[r], a);
            a = warp_sum(a);
            if (lane == 0) {
                const double nn = (i + 1 < m) ? sqrt(a) : 0.0;
                vn1[j] = nn;
                vn2[j] = nn;
            }
        } else if (lane == 0) {
            vn1[j] = nv * sqrt(tt);
        }
    }
}

// dorgqr: Q(:, c) for c < qc, Q = H_0 ... H_{k-1} [I; 0], applied backwards
__global__ void orgqr_step_kernel(const double *A, i64 lda, double *Q, i64 ldq, i64 m, int i, const double *tau) {
    __shared__ double sc[32];
    const int col = i + blockIdx.x;
    const double t = tau[i];
    double *x = Q + (i64)col * ldq;
    const double *v = A + (i64)i * lda;
    double part = 0.0;
    for (i64 r = i + 1 + threadIdx.x; r < m; r += blockDim.x) part = fma(v[r], x[r], part);
    const double w = block_sum(part, sc) + x[i];
    const double f = t * w;
    for (i64 r = i + 1 + threadIdx.x; r < m; r += blockDim.x) x[r] -= f * v[r];
    if (threadIdx.x == 0) x[i] -= f;
}

// ------------------------------------------------------------------ RSVDPACK rule
__global__ void sqnorm_kernel(const double *A, i64 ld, i64 m, int n, double *nrm, int *perm) {
    // serial order within each column, like get_matrix_column_norm_squared (MVF:407-418)
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        double a = 0.0;
        for (i64 r = 0; r < m; r++) a += A[r + j * ld] * A[r + j * ld];
        nrm[j] = a;
        perm[j] = j;
    }
}

__global__ void __launch_bounds__(1024) rsvdpack_select_kernel(double *R, i64 ld, i64 m, int n, int i, double *nrm,
                                                               int *perm, double *H, i64 ldh, PivCtl *ctl,
                                                               int tol_mode, double TOL, double zero_tol) {
    __shared__ double sc[32];
    if (ctl->stop) return;
    double bv;
    int pvt;
    // first index of the maximum squared norm: scan i..n-1 with strict '>' (RRA:1214-1222)
    block_argmax(nrm, i, n, bv, pvt);
    if (pvt >= n) pvt = i;
    if (i % 5 == 0) {
        double s = 0.0;
        if (tol_mode) {
            // serial sum in index order, like RRA:1239-1243
            if (threadIdx.x == 0) {
                for (int j = i; j < n; j++) s += nrm[j];
                s = sqrt(s) / n;
            }
        }
        if (threadIdx.x == 0) ctl->r22 = s;
    }
    __syncthreads();
    int stop = 0;
    if (threadIdx.x == 0) {
        // a vanished pivot column ends the factorisation: |norm| < 1e-10 (RRA:1250), or exactly
        // zero for the rank-only form (zero_tol = 0, RRA:1069)
        const bool vanished = zero_tol > 0.0 ? fabs(nrm[pvt]) < zero_tol : nrm[pvt] == 0.0;
        if (vanished && i > 0) stop = 1;
        else if (tol_mode && ctl->r22 < TOL) stop = 1;
        if (stop) ctl->stop = 1;
        else { ctl->frank = i + 1; ctl->pvt = pvt; }
        sc[0] = (double)stop;
    }
    __syncthreads();
    stop = (int)sc[0];
    __syncthreads();
    if (stop) return;
    if (pvt != i) {
        swap_columns(R, ld, m, pvt, i);
        if (threadIdx.x == 0) {
            const int t = perm[i]; perm[i] = perm[pvt]; perm[pvt] = t;
            const double u = nrm[pvt]; nrm[pvt] = nrm[i]; nrm[i] = u;
        }
    }
    __syncthreads();
    // h = x - |x| e_i on rows i..m-1, scaled so that |h|^2 = 2 (RRA:982-1004)
    double *h = H + (i64)i * ldh;
    double nx = 0.0;
    for (i64 r = i + threadIdx.x; r < m; r += blockDim.x) nx = fma(R[r + i * ld], R[r + i * ld], nx);
    nx = block_sum(nx, sc);
    const double normval = sqrt(nx);
    for (i64 r = threadIdx.x; r < m; r += blockDim.x) h[r] = (r >= i) ? R[r + i * ld] : 0.0;
    __syncthreads();
    if (threadIdx.x == 0) h[i] -= normval;
    __syncthreads();
    double hh = 0.0;
    for (i64 r = i + threadIdx.x; r < m; r += blockDim.x) hh = fma(h[r], h[r], hh);
    hh = block_sum(hh, sc);
    if (hh > 0.0) {
        const double scl = sqrt(2.0 / hh);
        for (i64 r = i + threadIdx.x; r < m; r += blockDim.x) h[r] *= scl;
    }
}

// R(:, j) -= h (h^T R(:, j)) for every column j (the reference updates all of R), then
// nrm[j] -= R(i,j)^2 for j > i.  One warp per column.
__global__ void rsvdpack_apply_kernel(double *R, i64 ld, i64 m, int n, int i, double *nrm, const double *H,
                                      i64 ldh, const PivCtl *ctl) {
    if (ctl->stop) return;
    const int lane = threadIdx.x & 31;
    const int j = (int)((blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5);
    if (j >= n) return;
    const double *h = H + (i64)i * ldh;
    double *x = R + (i64)j * ld;
    double w = 0.0;
    for (i64 r = i + lane; r < m; r += 32) w = fma(h[r], x[r], w);
    w = warp_sum(w);
    for (i64 r = i + lane; r < m; r += 32) x[r] -= h[r] * w;
    __syncwarp();
    if (lane == 0 && j > i) nrm[j] -= x[i] * x[i];
}

// Qk = H_0 ... H_{f-1} I(:, 0:f): backwards accumulation with the stored reflectors
__global__ void rsvdpack_formq_kernel(const double *H, i64 ldh, double *Q, i64 ldq, i64 m, int i) {
    __shared__ double sc[32];
    const int col = blockIdx.x;   // columns 0..f-1 (those < i are untouched: h is zero above i,
                                  // and rows >= i of e_col are zero for col < i)
    if (col < i) return;
    const double *h = H + (i64)i * ldh;
    double *x = Q + (i64)col * ldq;
    double part = 0.0;
    for (i64 r = i + threadIdx.x; r < m; r += blockDim.x) part = fma(h[r], x[r], part);
    const double w = block_sum(part, sc);
    for (i64 r = i + threadIdx.x; r < m; r += blockDim.x) x[r] -= h[r] * w;
}

// ------------------------------------------------------------------ LU solve (dgesv)
// Solves A X = B (n x n, n x nrhs) with partial pivoting; one 1024-thread block.
__global__ void __launch_bounds__(1024) lu_solve_kernel(double *A, i64 lda, double *B, i64 ldb, int n, int nrhs,
                                                        int *flag) {
    __shared__ int piv;
    for (int j = 0; j < n; j++) {
        if (threadIdx.x == 0) {
            int p = j;
            double best = fabs(A[j + (i64)j * lda]);
            for (int r = j + 1; r < n; r++) {
                const double v = fabs(A[r + (i64)j * lda]);
                if (v > best) { best = v; p = r; }
            }
            piv = p;
            if (best == 0.0) atomicExch(flag, 1);
        }
        __syncthreads();
        const int p = piv;
        if (p != j) {
            for (int c = threadIdx.x; c < n; c += blockDim.x) {
                const double t = A[j + (i64)c * lda]; A[j + (i64)c * lda] = A[p + (i64)c * lda]; A[p + (i64)c * lda] = t;
            }
            for (int c = threadIdx.x; c < nrhs; c += blockDim.x) {
                const double t = B[j + (i64)c * ldb]; B[j + (i64)c * ldb] = B[p + (i64)c * ldb]; B[p + (i64)c * ldb] = t;
            }
        }
        __syncthreads();
        const double d = A[j + (i64)j * lda];
        for (int r = j + 1 + threadIdx.x; r < n; r += blockDim.x) A[r + (i64)j * lda] /= d;
        __syncthreads();
        const int t = n - j - 1;
        for (i64 e = threadIdx.x; e < (i64)t * t; e += blockDim.x) {
            const int r = j + 1 + (int)(e % t), c = j + 1 + (int)(e / t);
            A[r + (i64)c * lda] -= A[r + (i64)j * lda] * A[j + (i64)c * lda];
        }
        for (i64 e = threadIdx.x; e < (i64)t * nrhs; e += blockDim.x) {
            const int r = j + 1 + (int)(e % t), c = (int)(e / t);
            B[r + (i64)c * ldb] -= A[r + (i64)j * lda] * B[j + (i64)c * ldb];
        }
        __syncthreads();
    }
    // back substitution, column-parallel
    for (int c = threadIdx.x; c < nrhs; c += blockDim.x) {
        double *b = B + (i64)c * ldb;
        for (int j = n - 1; j >= 0; j--) {
            double acc = b[j];
            for (int k = j + 1; k < n; k++) acc -= A[j + (i64)k * lda] * b[k];
            b[j] = acc / A[j + (i64)j * lda];
        }
    }
}

}  // namespace

void pivqr_lapack(cudaStream_t s, DM<double> A, double *d_tau, int *d_jpvt) {
    const i64 m = A.r;
    const int n = (int)A.c;
    const int kmin = (int)std::min<i64>(m, n);
    DBuf vb(sizeof(double) * 2 * std::max(1, n), s);
    double *vn1 = (double *)vb.get(), *vn2 = vn1 + n;
    colnorm_kernel<<<ceil_div(n, 8), 256, 0, s>>>(A.p, A.ld, m, n, vn1, vn2, d_jpvt);
    RSVD_LAUNCH_CK();
    const double tol3z = std::sqrt(std::ldexp(1.0, -53));   // sqrt(dlamch('Epsilon'))
    for (int i = 0; i < kmin; i++) {
        lapack_select_kernel<<<1, 1024, 0, s>>>(A.p, A.ld, m, n, i, vn1, vn2, d_jpvt, d_tau);
        const int ncols = n - i - 1;
        if (ncols > 0)
            lapack_apply_kernel<<<ceil_div((i64)ncols * 32, 256), 256, 0, s>>>(A.p, A.ld, m, n, i, d_tau, vn1, vn2, tol3z);
    }
    RSVD_LAUNCH_CK();
    ctx().launches += 2 * kmin + 1;
}

void form_q_from_reflectors(cudaStream_t s, DM<double> A, const double *d_tau, int nrefl, DM<double> Q) {
    set_identity(s, Q);
    for (int i = nrefl - 1; i >= 0; i--) {
        const int ncols = (int)Q.c - i;
        if (ncols > 0) orgqr_step_kernel<<<ncols, 256, 0, s>>>(A.p, A.ld, Q.p, Q.ld, Q.r, i, d_tau);
    }
    RSVD_LAUNCH_CK();
}

int pivqr_rsvdpack(cudaStream_t s, DM<double> R, DM<double> Qk, int k, double TOL, bool tol_mode, int *d_jpvt,
                   double zero_tol) {
    const i64 m = R.r;
    const int n = (int)R.c;
    DBuf nb(sizeof(double) * std::max(1, n), s);
    double *nrm = (double *)nb.get();
    DBuf cb(sizeof(PivCtl), s);
    PivCtl *ctl = (PivCtl *)cb.get();
    RSVD_CK(cudaMemsetAsync(ctl, 0, sizeof(PivCtl), s));
    DMat<double> H(m, std::max(1, k), s);
    sqnorm_kernel<<<ceil_div(n, 128), 128, 0, s>>>(R.p, R.ld, m, n, nrm, d_jpvt);
    for (int i = 0; i < k; i++) {
        rsvdpack_select_kernel<<<1, 1024, 0, s>>>(R.p, R.ld, m, n, i, nrm, d_jpvt, H.v.p, H.v.ld, ctl, tol_mode ? 1 : 0, TOL,
                                                    zero_tol);
        rsvdpack_apply_kernel<<<ceil_div((i64)n * 32, 256), 256, 0, s>>>(R.p, R.ld, m, n, i, nrm, H.v.p, H.v.ld, ctl);
    }
    RSVD_LAUNCH_CK();
    PivCtl h{};
    RSVD_CK(cudaMemcpyAsync(&h, ctl, sizeof(PivCtl), cudaMemcpyDeviceToHost, s));
    RSVD_CK(cudaStreamSynchronize(s));
    const int f = h.frank;
    if (Qk.p && f > 0) {
        DM<double> Qf = Qk.cols(0, f);
        set_identity(s, Qf);
        for (int i = f - 1; i >= 0; i--) rsvdpack_formq_kernel<<<f, 256, 0, s>>>(H.v.p, H.v.ld, Qf.p, Qf.ld, m, i);
        RSVD_LAUNCH_CK();
    }
    return f;
}

bool lu_solve(cudaStream_t s, DM<double> A, DM<double> B, int *d_flag) {
    RSVD_CK(cudaMemsetAsync(d_flag, 0, sizeof(int), s));
    lu_solve_kernel<<<1, 1024, 0, s>>>(A.p, A.ld, B.p, B.ld, (int)A.r, (int)B.c, d_flag);
    RSVD_LAUNCH_CK();
    int h = 0;
    RSVD_CK(cudaMemcpyAsync(&h, d_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    RSVD_CK(cudaStreamSynchronize(s));
    return h == 0;
}

}  // namespace rsvd
