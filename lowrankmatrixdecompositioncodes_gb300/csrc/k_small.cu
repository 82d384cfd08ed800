// k_small.cu -- the k x k (l x l) steps of every decomposition, templated on the compute
// type S: S = double in the FP64 mode (reproduces the reference), S = float in the mixed
// modes.  Storage is FP64 throughout; S only sets the arithmetic.
//
// Why two compute types: GB300 executes FP64 at ~2 FMA/clock/SM (cuBLAS DGEMM measures
// 1.1 TFLOP/s on the whole GPU), so an l x l factorisation that runs on one SM costs
// milliseconds in FP64 and tens of microseconds in FP32.  In the mixed modes the inputs
// of these steps (Grams of FP32 data) are only FP32-accurate anyway.
//
//   cholesky_small  : G = R^T R, one CTA; the upper triangle is kept packed in shared
//                     memory when it fits (else in global memory / L2)
//   tri_inv_upper   : Rinv = R^-1, one warp per column (back substitution), many SMs
//   jacobi_small    : one-sided Jacobi SVD, one CTA, round-robin pair ordering
#include "rsvd_internal.h"
#include "k_common.cuh"

#include <algorithm>
#include <cmath>
#include <limits>
#include <type_traits>

#include <cooperative_groups.h>

namespace rsvd {

namespace {

__host__ __device__ __forceinline__ long long pk(int i, int k) { return (long long)k * (k + 1) / 2 + i; }  // i <= k

template <typename S>
__device__ __forceinline__ S warp_sum_t(S v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ------------------------------------------------------------------ Cholesky
// Packed upper triangle P (column k holds rows 0..k).  Right-looking with deferred row
// scaling: step j updates the trailing triangle with P(j,i) P(j,k) / d_j (d_j the pivot)
// and leaves row j unscaled; rows are scaled by 1/sqrt(d_j) once at the end.  Two block
// barriers per step; the original diagonal (for the breakdown test) sits in shared memory.
template <typename S>
__global__ void __launch_bounds__(1024) chol_kernel(double *G, long long ldg, int n, double rel_tol, int *flag,
                                                    S *gbuf, int use_smem) {
    extern __shared__ __align__(16) unsigned char shraw[];
    S *P = use_smem ? (S *)shraw : gbuf;
    S *piv = use_smem ? (S *)(shraw + sizeof(S) * ((size_t)n * (n + 1) / 2)) : gbuf + (size_t)n * (n + 1) / 2;
    S *diag0 = piv + n;
    __shared__ int bad;
    __shared__ S inv_d;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) bad = 0;
    for (int k = wid; k < n; k += nw)
        for (int i = lane; i <= k; i += 32) P[pk(i, k)] = (S)G[i + (long long)k * ldg];
    for (int j = threadIdx.x; j < n; j += blockDim.x) diag0[j] = (S)G[j + (long long)j * ldg];
    __syncthreads();
    for (int j = 0; j < n; j++) {
        if (threadIdx.x == 0) {
            const S d = P[pk(j, j)];
            if (!(d > S(0)) || !isfinite((double)d) || !((double)d > rel_tol * (double)diag0[j])) { bad = 1; inv_d = S(0); }
            else inv_d = S(1) / d;
            piv[j] = d;
        }
        __syncthreads();
        if (bad) break;
        const S id = inv_d;
        for (int k = j + 1 + wid; k < n; k += nw) {
            const S f = P[pk(j, k)] * id;
            const long long ck = (long long)k * (k + 1) / 2;
            for (int i = j + 1 + lane; i <= k; i += 32) P[ck + i] -= P[pk(j, i)] * f;
        }
        __syncthreads();
    }
    if (bad) {
        if (threadIdx.x == 0) atomicExch(flag, 1);
        return;
    }
    for (long long e = threadIdx.x; e < (long long)n * n; e += blockDim.x) {
        const int i = (int)(e % n), k = (int)(e / n);
        double v = 0.0;
        if (i < k) v = (double)(P[pk(i, k)] / sqrt(piv[i]));
        else if (i == k) v = (double)sqrt(piv[i]);
        G[i + (long long)k * ldg] = v;
    }
}

// Blocked right-looking Cholesky on the packed upper triangle in shared memory (one CTA,
// 1024 threads, 32-column blocks):
//   A: warp 0 factors the diagonal block (unblocked, warp-synchronous);
//   B: the block row to its right, R_JK = R_JJ^-T G_JK, one warp per column (forward
//      substitution with the 32 rows of the column held one per lane);
//   C: trailing update G_IK -= R_JI^T R_JK over 32 x 32 tiles, 4 x 4 outputs per thread.
template <typename S>
__global__ void __launch_bounds__(1024) chol_blocked_kernel(double *G, long long ldg, int n, double rel_tol,
                                                            int *flag) {
    extern __shared__ __align__(16) unsigned char shraw[];
    S *P = (S *)shraw;
    S *diag0 = P + (size_t)n * (n + 1) / 2;
    __shared__ int bad;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) bad = 0;
    for (int k = wid; k < n; k += nw)
        for (int i = lane; i <= k; i += 32) P[pk(i, k)] = (S)G[i + (long long)k * ldg];
    for (int j = threadIdx.x; j < n; j += blockDim.x) diag0[j] = (S)G[j + (long long)j * ldg];
    __syncthreads();
    const int nb = (n + 31) / 32;
    for (int J = 0; J < nb; J++) {
        const int j0 = 32 * J, jw = min(32, n - j0);
        // ---- A: diagonal block in registers: lane t holds column j0+t (rows j0..j0+31);
        //      row j of R is broadcast from lane i's register c[j] by shuffles
        if (wid == 0) {
            S c[32];
            const long long ct = (long long)(j0 + lane) * (j0 + lane + 1) / 2 + j0;
#pragma unroll
            for (int i = 0; i < 32; i++) c[i] = (lane < jw && i <= lane) ? P[ct + i] : S(0);
            int bad_local = 0;
#pragma unroll
            for (int j = 0; j < 32; j++) {
                if (j < jw) {
                    const S d = __shfl_sync(0xffffffffu, c[j], j);
                    const bool ok = (d > S(0)) && isfinite(d) && (d > (S)rel_tol * diag0[j0 + j]);
                    bad_local |= !ok;
                    const S p = ok ? sqrt(d) : S(1);
                    const S inv = S(1) / p;
                    if (lane == j) c[j] = p;
                    else if (lane > j) c[j] *= inv;          // lane t now holds R(j, t)
#pragma unroll
                    for (int i = j + 1; i < 32; i++) {
                        const S rji = __shfl_sync(0xffffffffu, c[j], i);
                        if (lane >= i) c[i] -= rji * c[j];
                    }
                }
            }
            if (lane < jw) {
#pragma unroll
                for (int i = 0; i < 32; i++)
                    if (i <= lane) P[ct + i] = c[i];
            }
            if (lane == 0 && bad_local) bad = 1;
        }
        __syncthreads();
        if (bad) break;
        // ---- B: block row to the right, one warp per column
        S rdiag_inv = S(0);
        if (lane < jw) rdiag_inv = S(1) / P[pk(j0 + lane, j0 + lane)];
        const long long lrow = (long long)(j0 + lane) * (j0 + lane + 1) / 2 + j0;   // R(j0+t, j0+lane) = P[lrow + t]
        for (int k = j0 + jw + wid; k < n; k += nw) {
            const long long ck = (long long)k * (k + 1) / 2;
            S g = (lane < jw) ? P[ck + j0 + lane] : S(0);
            for (int t = 0; t < jw; t++) {
                S xt = (lane == t) ? g * rdiag_inv : S(0);
                xt = __shfl_sync(0xffffffffu, xt, t);
                if (lane == t) g = xt;
                else if (lane > t && lane < jw) g -= P[lrow + t] * xt;
            }
            if (lane < jw) P[ck + j0 + lane] = g;
        }
        __syncthreads();
        // ---- C: trailing update over tiles (I, K), J < I <= K, 4 x 4 per thread
        const int t0 = J + 1, nt = nb - t0;
        const int ntiles = nt * (nt + 1) / 2;
        const int sub = threadIdx.x & 63;             // 64 threads per tile: 8 x 8 threads x (4 x 4)
        const int tslot = threadIdx.x >> 6;           // 16 tiles in flight
        for (int tt = tslot; tt < ntiles; tt += 16) {
            // tile index -> (I, K) with I <= K
            int K = 0;
            while ((K + 1) * (K + 2) / 2 <= tt) K++;
            const int I = tt - K * (K + 1) / 2;
            const int ib = 32 * (t0 + I), kb = 32 * (t0 + K);
            const int ri = ib + (sub & 7) * 4, ck = kb + (sub >> 3) * 4;
            S acc[4][4];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = S(0);
            for (int t = 0; t < jw; t++) {
                const int row = j0 + t;
                S ra[4], rb[4];
#pragma unroll
                for (int a = 0; a < 4; a++) {
                    const int i = ri + a, k = ck + a;
                    ra[a] = (i < n) ? P[pk(row, i)] : S(0);
                    rb[a] = (k < n) ? P[pk(row, k)] : S(0);
                }
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int b = 0; b < 4; b++) acc[a][b] = fma(ra[a], rb[b], acc[a][b]);
            }
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    const int i = ri + a, k = ck + b;
                    if (i <= k && k < n) P[pk(i, k)] -= acc[a][b];
                }
        }
        __syncthreads();
    }
    if (bad) {
        if (threadIdx.x == 0) atomicExch(flag, 1);
        return;
    }
    for (long long e = threadIdx.x; e < (long long)n * n; e += blockDim.x) {
        const int i = (int)(e % n), k = (int)(e / n);
        G[i + (long long)k * ldg] = (i <= k) ? (double)P[pk(i, k)] : 0.0;
    }
}

// ------------------------------------------------------------------ triangular inverse
// Column c of X = R^-1 solves R x = e_c: back substitution from row c down to 0, the
// pending right-hand side kept in registers (rows spread over the 32 lanes).
template <typename S, int MAXR>
__global__ void tri_inv_kernel(const double *R, long long ldr, int n, double *X, long long ldx) {
    const int c = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= n) return;
    S b[MAXR];   // b[t] holds rhs row (lane + 32 t)
#pragma unroll
    for (int t = 0; t < MAXR; t++) {
        const int r = lane + 32 * t;
        b[t] = (r == c) ? S(1) : S(0);
    }
    double *x = X + (long long)c * ldx;
    for (int r = lane; r < n; r += 32) x[r] = 0.0;
    for (int j = c; j >= 0; j--) {
        const int owner = j & 31, slot = j >> 5;
        S bj = S(0);
#pragma unroll
        for (int t = 0; t < MAXR; t++)
            if (t == slot) bj = b[t];
        bj = __shfl_sync(0xffffffffu, bj, owner);
        const S xj = bj / (S)R[j + (long long)j * ldr];
        if (lane == 0) x[j] = (double)xj;
        // b[0..j-1] -= xj * R(0..j-1, j)
        const double *rc = R + (long long)j * ldr;
#pragma unroll
        for (int t = 0; t < MAXR; t++) {
            const int r = lane + 32 * t;
            if (r < j) b[t] -= xj * (S)rc[r];
        }
    }
}

// Shared-memory variant: CTA b solves columns [32b, 32b+32) (one warp each) against the
// packed upper triangle of R(0:cmax, 0:cmax) staged in shared memory.
template <typename S, int MAXR>
__global__ void __launch_bounds__(1024) tri_inv_smem_kernel(const double *R, long long ldr, int n, double *X,
                                                            long long ldx) {
    extern __shared__ __align__(16) unsigned char shraw[];
    S *Rs = (S *)shraw;
    const int cmax = min(n, (int)(blockIdx.x + 1) * 32);
    for (long long e = threadIdx.x; e < (long long)cmax * cmax; e += blockDim.x) {
        const int i = (int)(e % cmax), k = (int)(e / cmax);
        if (i <= k) Rs[pk(i, k)] = (S)R[i + (long long)k * ldr];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int c = blockIdx.x * 32 + (threadIdx.x >> 5);
    if (c >= n) return;
    S b[MAXR];
#pragma unroll
    for (int t = 0; t < MAXR; t++) b[t] = (lane + 32 * t == c) ? S(1) : S(0);
    double *x = X + (long long)c * ldx;
    for (int r = lane; r < n; r += 32) x[r] = 0.0;
    for (int j = c; j >= 0; j--) {
        const int owner = j & 31, slot = j >> 5;
        S bj = S(0);
#pragma unroll
        for (int t = 0; t < MAXR; t++)
            if (t == slot) bj = b[t];
        bj = __shfl_sync(0xffffffffu, bj, owner);
        const long long cj = (long long)j * (j + 1) / 2;
        const S xj = bj / Rs[cj + j];
        if (lane == 0) x[j] = (double)xj;
#pragma unroll
        for (int t = 0; t < MAXR; t++) {
            const int r = lane + 32 * t;
            if (r < j) b[t] -= xj * Rs[cj + r];
        }
    }
}

// ------------------------------------------------------------------ Jacobi SVD
__device__ __forceinline__ void rr_pair2(int np, int r, int i, int &a, int &b) {
    const int m = np - 1;
    if (i == 0) { a = 0; b = (r % m) + 1; }
    else { a = ((r + i) % m) + 1; b = ((r - i + m) % m) + 1; }
}

// W (n x n, compute type S, in global memory) is orthogonalised in place; V accumulates
// the rotations when non-null.  Converged when no pair has |w_p.w_q| > tol |w_p||w_q|.
template <typename S>
__global__ void __launch_bounds__(1024) jacobi_kernel_t(S *W, long long ldw, S *V, long long ldv, int n, S tol,
                                                        int max_sweeps, int *sweeps_out, int *flag) {
    __shared__ int rotated;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int np = n + (n & 1);
    int sweep = 0;
    for (; sweep < max_sweeps; sweep++) {
        if (threadIdx.x == 0) rotated = 0;
        __syncthreads();
        for (int r = 0; r < np - 1; r++) {
            for (int pi = wid; pi < np / 2; pi += nw) {
                int p, q;
                rr_pair2(np, r, pi, p, q);
                if (p >= n || q >= n) continue;
                if (p > q) { const int t = p; p = q; q = t; }
                S *wp = W + (long long)p * ldw, *wq = W + (long long)q * ldw;
                S a = 0, b = 0, d = 0;
                for (int i = lane; i < n; i += 32) {
                    const S x = wp[i], y = wq[i];
                    a = fma(x, x, a); b = fma(y, y, b); d = fma(x, y, d);
                }
                a = warp_sum_t(a); b = warp_sum_t(b); d = warp_sum_t(d);
                if (d == S(0) || fabs(d) <= tol * sqrt(a * b)) continue;
                const S zeta = (b - a) / (S(2) * d);
                const S t = copysign(S(1), zeta) / (fabs(zeta) + sqrt(S(1) + zeta * zeta));
                const S cs = S(1) / sqrt(S(1) + t * t), sn = cs * t;
                for (int i = lane; i < n; i += 32) {
                    const S x = wp[i], y = wq[i];
                    wp[i] = cs * x - sn * y;
                    wq[i] = sn * x + cs * y;
                }
                if (V) {
                    S *vp = V + (long long)p * ldv, *vq = V + (long long)q * ldv;
                    for (int i = lane; i < n; i += 32) {
                        const S x = vp[i], y = vq[i];
                        vp[i] = cs * x - sn * y;
                        vq[i] = sn * x + cs * y;
                    }
                }
                if (lane == 0) rotated = 1;
            }
            __syncthreads();
        }
        const int any = rotated;
        __syncthreads();
        if (!any) break;
    }
    if (threadIdx.x == 0) {
        *sweeps_out = sweep;
        if (sweep >= max_sweeps) atomicExch(flag, 1);
    }
}

// Cluster version: CL CTAs (one cluster) split the n rows of W and V; every CTA keeps its
// rows of both in shared memory (column-major, rows_per rows).  Per round:
//   phase 1: partial (|w_p|^2, |w_q|^2, w_p.w_q) over the local rows for every pair, pushed
//            into the partial buffer of EVERY CTA of the cluster (remote shared stores);
//   cluster barrier (release/acquire) ;
//   phase 2: each CTA sums the CL partials in rank order (identical in all CTAs, so all
//            take identical rotation decisions) and rotates its local rows of W and V.
// Partials are double-buffered by round parity: a CTA cannot overwrite a buffer before
// every CTA has passed the next barrier, i.e. finished reading it.
template <typename S, int CL>
__global__ void __launch_bounds__(1024) jacobi_cluster_kernel(const double *G, long long ldg, int n, int rows_per,
                                                              S tol, int max_sweeps, S *Wout, S *Vout, long long ldo,
                                                              int *sweeps_out, int *flag) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    extern __shared__ __align__(16) unsigned char shraw[];
    const int np = n + (n & 1), npairs = np / 2;
    S *Wl = (S *)shraw;                                   // n columns x rows_per
    S *Vl = Wl + (size_t)n * rows_per;
    S *part = Vl + (size_t)n * rows_per;                  // [2][CL][3 * npairs]
    __shared__ int rotated;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int r0 = rank * rows_per, nloc = max(0, min(n, r0 + rows_per) - r0);
    for (long long e = threadIdx.x; e < (long long)n * rows_per; e += blockDim.x) {
        const int c = (int)(e / rows_per), rr = (int)(e % rows_per);
        const int gr = r0 + rr;
        Wl[e] = (rr < nloc) ? (S)G[gr + (long long)c * ldg] : S(0);
        Vl[e] = (rr < nloc && gr == c) ? S(1) : S(0);
    }
    cluster.sync();
    int sweep = 0, round = 0;
    for (; sweep < max_sweeps; sweep++) {
        if (threadIdx.x == 0) rotated = 0;
        for (int r = 0; r < np - 1; r++, round++) {
            const int buf = round & 1;
            // phase 1
            for (int pi = wid; pi < npairs; pi += nw) {
                int p, q;
                rr_pair2(np, r, pi, p, q);
                if (p > q) { const int t = p; p = q; q = t; }   // same order as phase 2
                S a = 0, b = 0, d = 0;
                if (p < n && q < n) {
                    const S *wp = Wl + (size_t)p * rows_per, *wq = Wl + (size_t)q * rows_per;
                    for (int i = lane; i < nloc; i += 32) {
                        const S x = wp[i], y = wq[i];
                        a = fma(x, x, a); b = fma(y, y, b); d = fma(x, y, d);
                    }
                    a = warp_sum_t(a); b = warp_sum_t(b); d = warp_sum_t(d);
                }
                if (lane < CL) {
                    S *dst = cluster.map_shared_rank(part, lane);
                    S *slot = dst + ((size_t)buf * CL + rank) * 3 * npairs + 3 * pi;
                    slot[0] = a; slot[1] = b; slot[2] = d;
                }
            }
            cluster.sync();
            // phase 2
            for (int pi = wid; pi < npairs; pi += nw) {
                int p, q;
                rr_pair2(np, r, pi, p, q);
                if (p >= n || q >= n) continue;
                if (p > q) { const int t = p; p = q; q = t; }
                S a = 0, b = 0, d = 0;
#pragma unroll
                for (int src = 0; src < CL; src++) {
                    const S *slot = part + ((size_t)buf * CL + src) * 3 * npairs + 3 * pi;
                    a += slot[0]; b += slot[1]; d += slot[2];
                }
                if (d == S(0) || fabs(d) <= tol * sqrt(a * b)) continue;
                const S zeta = (b - a) / (S(2) * d);
                const S t = copysign(S(1), zeta) / (fabs(zeta) + sqrt(S(1) + zeta * zeta));
                const S cs = S(1) / sqrt(S(1) + t * t), sn = cs * t;
                S *wp = Wl + (size_t)p * rows_per, *wq = Wl + (size_t)q * rows_per;
                S *vp = Vl + (size_t)p * rows_per, *vq = Vl + (size_t)q * rows_per;
                for (int i = lane; i < nloc; i += 32) {
                    const S x = wp[i], y = wq[i];
                    wp[i] = cs * x - sn * y;
                    wq[i] = sn * x + cs * y;
                    const S u = vp[i], v = vq[i];
                    vp[i] = cs * u - sn * v;
                    vq[i] = sn * u + cs * v;
                }
                if (lane == 0) rotated = 1;
            }
            __syncthreads();
        }
        const int any = rotated;
        __syncthreads();
        if (!any) break;
    }
    for (long long e = threadIdx.x; e < (long long)n * rows_per; e += blockDim.x) {
        const int c = (int)(e / rows_per), rr = (int)(e % rows_per);
        if (rr < nloc) {
            Wout[r0 + rr + (long long)c * ldo] = Wl[e];
            Vout[r0 + rr + (long long)c * ldo] = Vl[e];
        }
    }
    if (rank == 0 && threadIdx.x == 0) {
        *sweeps_out = sweep;
        if (sweep >= max_sweeps) atomicExch(flag, 1);
    }
    cluster.sync();   // no CTA leaves while a peer may still write into its shared memory
}

// Block-cyclic one-sided Jacobi on a cluster of 8 CTAs.  The n columns of W and V are
// cut into 16 blocks of bs columns.  CTA i holds the blocks at tournament positions i
// (slot 0) and 15-i (slot 1), whole columns (all n rows) of W and V, in shared memory.
// A super-round orthogonalises every pair among the CTA's 2*bs columns (one cyclic inner
// sweep, block barriers only); then positions 1..15 rotate by one (position 0 stays) and
// every block moves to its next holder through distributed shared memory, followed by
// one cluster barrier.  15 super-rounds meet every pair of blocks once: one outer sweep.
// Outer sweeps repeat until no CTA rotated anything during a whole sweep.
// Shared memory per CTA: 2 buffers x 2 slots x bs x ldr x 2 (W, V) x sizeof(S).
template <typename S>
__global__ void __launch_bounds__(1024) jacobi_block_cluster_kernel(const double *G, long long ldg, int n, int bs,
                                                                    int ldr, S tol, int max_sweeps, S *Wout, S *Vout,
                                                                    long long ldo, int *sweeps_out, int *flag) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    constexpr int CLN = 8, NBLK = 16;
    extern __shared__ __align__(16) unsigned char shraw[];
    const size_t slot_elems = (size_t)bs * ldr * 2;          // W columns then V columns
    S *buf = (S *)shraw;                                      // [2 buffers][2 slots][slot_elems]
    __shared__ int blk[2][2];                                 // block id held in [buffer][slot]
    __shared__ int rot_count;
    __shared__ int sweep_rot[CLN];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    auto slot_ptr = [&](S *base, int b, int sl) { return base + ((size_t)b * 2 + sl) * slot_elems; };
    auto col_w = [&](S *sp, int j) { return sp + (size_t)j * ldr; };
    auto col_v = [&](S *sp, int j) { return sp + (size_t)(bs + j) * ldr; };

    // initial placement: slot 0 <- block rank, slot 1 <- block 15 - rank
    if (threadIdx.x == 0) {
        blk[0][0] = rank;
        blk[0][1] = NBLK - 1 - rank;
        rot_count = 0;
    }
    for (int sl = 0; sl < 2; sl++) {
        const int b = (sl == 0) ? rank : NBLK - 1 - rank;
        S *sp = slot_ptr(buf, 0, sl);
        for (long long e = threadIdx.x; e < (long long)bs * ldr; e += blockDim.x) {
            const int j = (int)(e / ldr), r = (int)(e % ldr);
            const int c = b * bs + j;
            const bool ok = (c < n && r < n);
            col_w(sp, j)[r] = ok ? (S)G[r + (long long)c * ldg] : S(0);
            col_v(sp, j)[r] = (ok && r == c) ? S(1) : S(0);
        }
    }
    cluster.sync();
    int cur = 0, sweep = 0;
    const int nloc = 2 * bs;                 // local columns (even)
    for (; sweep < max_sweeps; sweep++) {
        for (int sr = 0; sr < NBLK - 1; sr++) {
            S *s0 = slot_ptr(buf, cur, 0), *s1 = slot_ptr(buf, cur, 1);
            const int b0 = blk[cur][0], b1 = blk[cur][1];
            // ---- super-round 0 of a sweep: full cyclic sweep over the 2*bs local columns
            //      (covers the pairs inside every block once per sweep); later super-rounds:
            //      only the bs x bs cross pairs of the two blocks, bs rounds of bs pairs
            const bool full = (sr == 0);
            const int nrounds = full ? nloc - 1 : bs;
            for (int r = 0; r < nrounds; r++) {
                for (int pi = wid; pi < (full ? nloc / 2 : bs); pi += nw) {
                    int p, q;
                    if (full) {
                        rr_pair2(nloc, r, pi, p, q);
                        if (p > q) { const int t = p; p = q; q = t; }
                    } else {
                        p = pi;
                        q = bs + (pi + r) % bs;
                    }
                    // skip padding columns beyond n
                    const int gp = (p < bs) ? b0 * bs + p : b1 * bs + (p - bs);
                    const int gq = (q < bs) ? b0 * bs + q : b1 * bs + (q - bs);
                    if (gp >= n || gq >= n) continue;
                    S *wp = (p < bs) ? col_w(s0, p) : col_w(s1, p - bs);
                    S *wq = (q < bs) ? col_w(s0, q) : col_w(s1, q - bs);
                    // columns are zero beyond n up to ldr (a multiple of 4), so whole
                    // 16-byte vectors can be processed: VW elements per lane per access
                    constexpr int VW = 16 / sizeof(S);
                    using V16 = typename std::conditional<sizeof(S) == 4, float4, double2>::type;
                    const int nvec = ldr / VW;
                    S a = 0, b = 0, d = 0;
                    for (int iv = lane; iv < nvec; iv += 32) {
                        const V16 xv = reinterpret_cast<const V16 *>(wp)[iv];
                        const V16 yv = reinterpret_cast<const V16 *>(wq)[iv];
                        const S *x = reinterpret_cast<const S *>(&xv), *y = reinterpret_cast<const S *>(&yv);
#pragma unroll
                        for (int e = 0; e < VW; e++) {
                            a = fma(x[e], x[e], a); b = fma(y[e], y[e], b); d = fma(x[e], y[e], d);
                        }
                    }
                    a = warp_sum_t(a); b = warp_sum_t(b); d = warp_sum_t(d);
                    if (d == S(0) || fabs(d) <= tol * sqrt(a * b)) continue;
                    const S zeta = (b - a) / (S(2) * d);
                    const S t = copysign(S(1), zeta) / (fabs(zeta) + sqrt(S(1) + zeta * zeta));
                    const S cs = S(1) / sqrt(S(1) + t * t), sn = cs * t;
                    S *vp = (p < bs) ? col_v(s0, p) : col_v(s1, p - bs);
                    S *vq = (q < bs) ? col_v(s0, q) : col_v(s1, q - bs);
                    for (int iv = lane; iv < nvec; iv += 32) {
                        V16 xv = reinterpret_cast<V16 *>(wp)[iv], yv = reinterpret_cast<V16 *>(wq)[iv];
                        V16 uv = reinterpret_cast<V16 *>(vp)[iv], vv = reinterpret_cast<V16 *>(vq)[iv];
                        S *x = reinterpret_cast<S *>(&xv), *y = reinterpret_cast<S *>(&yv);
                        S *u = reinterpret_cast<S *>(&uv), *v = reinterpret_cast<S *>(&vv);
#pragma unroll
                        for (int e = 0; e < VW; e++) {
                            const S x0 = x[e], y0 = y[e], u0 = u[e], v0 = v[e];
                            x[e] = cs * x0 - sn * y0;
                            y[e] = sn * x0 + cs * y0;
                            u[e] = cs * u0 - sn * v0;
                            v[e] = sn * u0 + cs * v0;
                        }
                        reinterpret_cast<V16 *>(wp)[iv] = xv;
                        reinterpret_cast<V16 *>(wq)[iv] = yv;
                        reinterpret_cast<V16 *>(vp)[iv] = uv;
                        reinterpret_cast<V16 *>(vq)[iv] = vv;
                    }
                    if (lane == 0) atomicAdd(&rot_count, 1);
                }
                __syncthreads();
            }
            // ---- move blocks to their next holders (positions 1..15 rotate by one)
            const int nxt = cur ^ 1;
            int dst0, dsl0, dst1, dsl1;       // destination (cta, slot) of local slots 0 and 1
            if (rank == 0) { dst0 = 0; dsl0 = 0; }
            else if (rank < CLN - 1) { dst0 = rank + 1; dsl0 = 0; }
            else { dst0 = CLN - 1; dsl0 = 1; }
            if (rank == 0) { dst1 = 1; dsl1 = 0; }
            else { dst1 = rank - 1; dsl1 = 1; }
            for (int sl = 0; sl < 2; sl++) {
                const int dc = sl ? dst1 : dst0, ds = sl ? dsl1 : dsl0;
                S *src = slot_ptr(buf, cur, sl);
                S *dst = cluster.map_shared_rank(slot_ptr(buf, nxt, ds), dc);
                const size_t nvec = slot_elems * sizeof(S) / 16;
                const float4 *s4 = (const float4 *)src;
                float4 *d4 = (float4 *)dst;
                for (size_t e = threadIdx.x; e < nvec; e += blockDim.x) d4[e] = s4[e];
                if (threadIdx.x == 0) {
                    int *rb = cluster.map_shared_rank(&blk[nxt][ds], dc);
                    *rb = sl ? b1 : b0;
                }
            }
            cluster.sync();
            cur = nxt;
        }
        // ---- did any CTA rotate during this sweep?
        if (threadIdx.x < CLN) {
            int *dstf = cluster.map_shared_rank(&sweep_rot[rank], (unsigned)threadIdx.x);
            *dstf = rot_count;
        }
        cluster.sync();
        int total = 0;
#pragma unroll
        for (int c = 0; c < CLN; c++) total += sweep_rot[c];
        __syncthreads();
        if (threadIdx.x == 0) rot_count = 0;
        cluster.sync();
        if (total == 0) break;
    }
    // ---- write the columns this CTA holds
    for (int sl = 0; sl < 2; sl++) {
        S *sp = slot_ptr(buf, cur, sl);
        const int b = blk[cur][sl];
        for (long long e = threadIdx.x; e < (long long)bs * n; e += blockDim.x) {
            const int j = (int)(e / n), r = (int)(e % n);
            const int c = b * bs + j;
            if (c < n) {
                Wout[r + (long long)c * ldo] = col_w(sp, j)[r];
                Vout[r + (long long)c * ldo] = col_v(sp, j)[r];
            }
        }
    }
    if (rank == 0 && threadIdx.x == 0) {
        *sweeps_out = sweep;
        if (sweep >= max_sweeps) atomicExch(flag, 1);
    }
    cluster.sync();
}

template <typename S>
__global__ void colnorm_kernel_t(const S *W, long long ldw, int n, double *sv) {
    const int lane = threadIdx.x & 31;
    for (int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); j < n; j += gridDim.x * (blockDim.x >> 5)) {
        double a = 0;
        for (int i = lane; i < n; i += 32) a = fma((double)W[i + (long long)j * ldw], (double)W[i + (long long)j * ldw], a);
        a = warp_sum(a);
        if (lane == 0) sv[j] = sqrt(a);
    }
}
__global__ void rank_desc_kernel(const double *sv, int n, int *rank) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double v = sv[j];
    int r = 0;
    for (int i = 0; i < n; i++) r += (sv[i] > v) || (sv[i] == v && i < j);
    rank[j] = r;
}
// U(:, rank j) = W(:, j) / sv_j ; V(:, rank j) = Vacc(:, j)  (or, without Vacc, left for the caller)
template <typename S>
__global__ void scatter_kernel_t(const S *W, long long ldw, const S *Vin, long long ldvi, const double *sv,
                                 const int *rank, int n, double *U, long long ldu, double *V, long long ldv,
                                 double *sv_sorted) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)n * n;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        const int r = rank[j];
        const double s = sv[j];
        U[i + (long long)r * ldu] = (s > 0.0) ? (double)W[i + j * ldw] / s : 0.0;
        if (Vin) V[i + (long long)r * ldv] = (double)Vin[i + j * ldvi];
        if (i == 0) sv_sorted[r] = s;
    }
}
template <typename S>
__global__ void load_kernel_t(const double *G, long long ldg, S *W, long long ldw, int n, int identity_to) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)n * n;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        W[i + (long long)j * ldw] = identity_to ? (S)(i == j ? 1.0 : 0.0) : (S)G[i + (long long)j * ldg];
    }
}

unsigned gfor(long long n) {
    long long g = (n + 255) / 256;
    return (unsigned)std::max<long long>(1, std::min<long long>(g, (long long)std::max(1, ctx().sms) * 8));
}

}  // namespace

template <typename S>
bool cholesky_small(cudaStream_t s, DM<double> G, double rel_tol, int *d_flag) {
    const int n = (int)G.r;
    if (G.r != G.c) fail(RSVD_ERR_ARGUMENT, "cholesky: not square");
    if (n == 0) return true;
    RSVD_CK(cudaMemsetAsync(d_flag, 0, sizeof(int), s));
    const size_t bpacked = sizeof(S) * ((size_t)n * (n + 1) / 2 + (size_t)n);
    if (bpacked <= 220 * 1024) {
        auto kb = chol_blocked_kernel<S>;
        RSVD_CK(cudaFuncSetAttribute(kb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(bpacked, 1024)));
        kb<<<1, 1024, std::max<size_t>(bpacked, 1024), s>>>(G.p, G.ld, n, rel_tol, d_flag);
        RSVD_LAUNCH_CK();
        ctx().launches++;
        int hb = 0;
        RSVD_CK(cudaMemcpyAsync(&hb, d_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
        RSVD_CK(cudaStreamSynchronize(s));
        return hb == 0;
    }
    const size_t packed = sizeof(S) * ((size_t)n * (n + 1) / 2 + 2 * (size_t)n);
    const bool smem = packed <= 200 * 1024;
    DBuf gb(smem ? 16 : packed, s);
    auto k = chol_kernel<S>;
    if (smem && packed > 48 * 1024)
        RSVD_CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)packed));
    k<<<1, 1024, smem ? packed : 0, s>>>(G.p, G.ld, n, rel_tol, d_flag, (S *)gb.get(), smem ? 1 : 0);
    RSVD_LAUNCH_CK();
    ctx().launches++;
    int h = 0;
    RSVD_CK(cudaMemcpyAsync(&h, d_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    RSVD_CK(cudaStreamSynchronize(s));
    return h == 0;
}
template bool cholesky_small<double>(cudaStream_t, DM<double>, double, int *);
template bool cholesky_small<float>(cudaStream_t, DM<double>, double, int *);

template <typename S>
void tri_inv_upper(cudaStream_t s, DM<double> R, DM<double> X) {
    const int n = (int)R.r;
    if (n == 0) return;
    const size_t sm = sizeof(S) * (size_t)n * (n + 1) / 2;
    if (sm <= 200 * 1024 && n <= 512) {
        const unsigned nb = (unsigned)((n + 31) / 32);
        if (n <= 256) {
            auto k = tri_inv_smem_kernel<S, 8>;
            RSVD_CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(sm, 1024)));
            k<<<nb, 1024, std::max<size_t>(sm, 1024), s>>>(R.p, R.ld, n, X.p, X.ld);
        } else {
            auto k = tri_inv_smem_kernel<S, 16>;
            RSVD_CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            k<<<nb, 1024, sm, s>>>(R.p, R.ld, n, X.p, X.ld);
        }
        RSVD_LAUNCH_CK();
        ctx().launches++;
        return;
    }
    const long long threads = (long long)n * 32;
    const unsigned blocks = (unsigned)((threads + 127) / 128);
    if (n <= 256) tri_inv_kernel<S, 8><<<blocks, 128, 0, s>>>(R.p, R.ld, n, X.p, X.ld);
    else if (n <= 512) tri_inv_kernel<S, 16><<<blocks, 128, 0, s>>>(R.p, R.ld, n, X.p, X.ld);
    else if (n <= 1024) tri_inv_kernel<S, 32><<<blocks, 128, 0, s>>>(R.p, R.ld, n, X.p, X.ld);
    else if (n <= 4096) tri_inv_kernel<S, 128><<<blocks, 128, 0, s>>>(R.p, R.ld, n, X.p, X.ld);
    else fail(RSVD_ERR_ARGUMENT, "tri_inv_upper: order above 4096");
    RSVD_LAUNCH_CK();
    ctx().launches++;
}
template void tri_inv_upper<double>(cudaStream_t, DM<double>, DM<double>);
template void tri_inv_upper<float>(cudaStream_t, DM<double>, DM<double>);

template <typename S>
int jacobi_small(cudaStream_t s, DM<double> G, DM<double> U, DM<double> V, double *d_sv, int *d_flag) {
    const int n = (int)G.r;
    if (G.r != G.c) fail(RSVD_ERR_ARGUMENT, "jacobi: not square");
    if (n == 0) return 0;
    const long long ld = pad_ld(n);
    DBuf wb(sizeof(S) * (size_t)ld * n, s), vb(sizeof(S) * (size_t)ld * n, s);
    S *W = (S *)wb.get(), *Vacc = (S *)vb.get();
    DBuf aux(sizeof(int) * (n + 2), s);
    int *d_sweeps = (int *)aux.get(), *d_rank = d_sweeps + 2;
    DBuf svb(sizeof(double) * n, s);
    double *d_raw = (double *)svb.get();
    const S tol = (S)(4.0 * std::sqrt((double)n) * (double)std::numeric_limits<S>::epsilon());
    RSVD_CK(cudaMemsetAsync(d_flag, 0, sizeof(int), s));
    constexpr int CL = 8;
    const int rows_per = (n + CL - 1) / CL;
    const int npairs = (n + (n & 1)) / 2;
    const size_t csmem = sizeof(S) * ((size_t)2 * n * rows_per + (size_t)2 * CL * 3 * npairs);
    const int bs = (n + 15) / 16, ldr = (n + 3) / 4 * 4;
    const size_t bsmem = sizeof(S) * (size_t)4 * bs * ldr * 2;
    cudaLaunchAttribute cattr[1];
    cattr[0].id = cudaLaunchAttributeClusterDimension;
    cattr[0].val.clusterDim.x = CL;
    cattr[0].val.clusterDim.y = 1;
    cattr[0].val.clusterDim.z = 1;
    if (bsmem <= 220 * 1024 && n >= 64) {
        auto kern = jacobi_block_cluster_kernel<S>;
        RSVD_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bsmem));
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(CL);
        cfg.blockDim = dim3(1024);
        cfg.dynamicSmemBytes = bsmem;
        cfg.stream = s;
        cfg.attrs = cattr;
        cfg.numAttrs = 1;
        RSVD_CK(cudaLaunchKernelEx(&cfg, kern, (const double *)G.p, (long long)G.ld, n, bs, ldr, tol, 40, W, Vacc,
                                   (long long)ld, d_sweeps, d_flag));
    } else if (csmem <= 200 * 1024 && n >= 64) {
        auto kern = jacobi_cluster_kernel<S, CL>;
        RSVD_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csmem));
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(CL);
        cfg.blockDim = dim3(1024);
        cfg.dynamicSmemBytes = csmem;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = CL;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        RSVD_CK(cudaLaunchKernelEx(&cfg, kern, (const double *)G.p, (long long)G.ld, n, rows_per, tol, 40, W, Vacc,
                                   (long long)ld, d_sweeps, d_flag));
    } else {
        load_kernel_t<S><<<gfor((long long)n * n), 256, 0, s>>>(G.p, G.ld, W, ld, n, 0);
        load_kernel_t<S><<<gfor((long long)n * n), 256, 0, s>>>(G.p, G.ld, Vacc, ld, n, 1);
        jacobi_kernel_t<S><<<1, 1024, 0, s>>>(W, ld, Vacc, ld, n, tol, 40, d_sweeps, d_flag);
    }
    colnorm_kernel_t<S><<<ceil_div(n, 8), 256, 0, s>>>(W, ld, n, d_raw);
    rank_desc_kernel<<<ceil_div(n, 256), 256, 0, s>>>(d_raw, n, d_rank);
    scatter_kernel_t<S><<<gfor((long long)n * n), 256, 0, s>>>(W, ld, Vacc, ld, d_raw, d_rank, n, U.p, U.ld, V.p, V.ld,
                                                                 d_sv);
    RSVD_LAUNCH_CK();
    ctx().launches += 6;
    int sweeps = 0;
    RSVD_CK(cudaMemcpyAsync(&sweeps, d_sweeps, sizeof(int), cudaMemcpyDeviceToHost, s));
    RSVD_CK(cudaStreamSynchronize(s));
    if (ctx().opts.verbose) std::fprintf(stderr, "rsvdpack: jacobi n=%d (%s) sweeps=%d\n", n, sizeof(S) == 4 ? "fp32" : "fp64", sweeps);
    return sweeps;
}
template int jacobi_small<double>(cudaStream_t, DM<double>, DM<double>, DM<double>, double *, int *);
template int jacobi_small<float>(cudaStream_t, DM<double>, DM<double>, DM<double>, double *, int *);

}  // namespace rsvd
