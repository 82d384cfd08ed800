// k_chol.cu -- the triangular l x l steps of CholeskyQR / CholeskyQR2 on 32 x 32 tiles:
//
//   chol_factor<S>    G = R^T R (upper R), right-looking blocked Cholesky.  Each step
//                     factors the diagonal tile in one warp and inverts it by back
//                     substitution, so the panel R_JK = R_JJ^-T G_JK and the trailing update
//                     G_IK -= R_JI^T R_JK are plain tile products (one warp per tile).
//                     Orders up to 288 (FP32) / 192 (FP64) run in one CTA with every
//                     tile resident in shared memory; larger orders run one launch per
//                     panel and per trailing update over tiles in global memory (L2).
//   tri_inv_tiles     X = R^-1 from R and the inverted diagonal tiles: one CTA per block
//                     column, X_IJ = -R_II^-1 sum_{K=I+1..J} R_IK X_KJ from I = J-1 down.
//   trsm_right_tiles  Q = Y R^-1 for tall Y: one CTA per slab of rows solves Q R = Y by
//                     block columns, the slab's Q resident in shared memory.
//   tri_mul_upper     C = A B for upper-triangular A, B (the R2 R1 of CholeskyQR2).
//
// Compute type S: float in the mixed-precision modes, double in the FP64 mode; the
// l x l matrices are stored in FP64 at the interface.  The factorisation follows the
// semantics of the Householder-based QR it replaces in the reference's range finder
// (QR_factorization_getQ, matrix_vector_functions_intel_mkl.c:1251-1263): the R factor
// of Y is the Cholesky factor of Y^T Y.
#include "rsvd_internal.h"
#include "k_common.cuh"

#include <algorithm>
#include <cmath>
#include <type_traits>

namespace rsvd {

namespace {

constexpr int TB = 32;            // tile order
constexpr int TP = 36;            // row pitch of a tile in shared memory (16-byte rows)
constexpr int TE = TB * TP;       // shared-memory elements per tile
constexpr unsigned FULL = 0xffffffffu;

__host__ __device__ __forceinline__ int tix(int I, int K) { return K * (K + 1) / 2 + I; }   // I <= K

// (I, K) of packed upper tile index t
__device__ __forceinline__ void untix(int t, int &I, int &K) {
    int k = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
    while (k * (k + 1) / 2 > t) k--;
    while ((k + 1) * (k + 2) / 2 <= t) k++;
    K = k;
    I = t - k * (k + 1) / 2;
}

// Lane -> 4 x 8 block of a 32 x 32 tile: rows r0..r0+3, columns c0..c0+7.
__device__ __forceinline__ int lane_r0() { return ((threadIdx.x & 31) >> 2) * 4; }
__device__ __forceinline__ int lane_c0() { return ((threadIdx.x & 31) & 3) * 8; }

template <typename S>
__device__ __forceinline__ void ld4(const S *p, S (&o)[4]) {
    if constexpr (sizeof(S) == 4) {
        const float4 v = *reinterpret_cast<const float4 *>(p);
        o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
    } else {
        const double2 a = *reinterpret_cast<const double2 *>(p), b = *reinterpret_cast<const double2 *>(p + 2);
        o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
    }
}

template <typename S>
__device__ __forceinline__ void zero_acc(S (&acc)[4][8]) {
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 8; b++) acc[a][b] = S(0);
}

// acc(r, c) += sum_{k0 <= k < k1} P[k][r] Q[k][c]     (P^T Q, row-major tiles of pitch TP)
// FP32: packed pairs of adjacent columns (FFMA2), P's value broadcast; same rounding as fma.
template <typename S>
__device__ __forceinline__ void tile_tn(const S *P, const S *Q, int k0, int k1, S (&acc)[4][8]) {
    const int r0 = lane_r0(), c0 = lane_c0();
    if constexpr (sizeof(S) == 4) {
        float2 acc2[4][4];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) acc2[a][b] = make_float2(acc[a][2 * b], acc[a][2 * b + 1]);
        for (int k = k0; k < k1; k++) {
            const float4 p4 = *reinterpret_cast<const float4 *>(P + k * TP + r0);
            const float4 qa = *reinterpret_cast<const float4 *>(Q + k * TP + c0);
            const float4 qb = *reinterpret_cast<const float4 *>(Q + k * TP + c0 + 4);
            const float pv[4] = {p4.x, p4.y, p4.z, p4.w};
            const float2 qp[4] = {make_float2(qa.x, qa.y), make_float2(qa.z, qa.w), make_float2(qb.x, qb.y),
                                  make_float2(qb.z, qb.w)};
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const float2 pp = make_float2(pv[a], pv[a]);
#pragma unroll
                for (int b = 0; b < 4; b++) acc2[a][b] = __ffma2_rn(pp, qp[b], acc2[a][b]);
            }
        }
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) {
                acc[a][2 * b] = acc2[a][b].x;
                acc[a][2 * b + 1] = acc2[a][b].y;
            }
    } else {
        for (int k = k0; k < k1; k++) {
            S p[4], q[8], q2[4];
            ld4<S>(P + k * TP + r0, p);
            ld4<S>(Q + k * TP + c0, *reinterpret_cast<S(*)[4]>(q));
            ld4<S>(Q + k * TP + c0 + 4, q2);
#pragma unroll
            for (int b = 0; b < 4; b++) q[4 + b] = q2[b];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 8; b++) acc[a][b] = fma(p[a], q[b], acc[a][b]);
        }
    }
}

// acc(r, c) += sum_{k0 <= k < k1} P[r][k] Q[k][c]     (P Q)
template <typename S>
__device__ __forceinline__ void tile_nn(const S *P, const S *Q, int k0, int k1, S (&acc)[4][8]) {
    const int r0 = lane_r0(), c0 = lane_c0();
    for (int k = k0; k < k1; k++) {
        S p[4], q[8], q2[4];
#pragma unroll
        for (int a = 0; a < 4; a++) p[a] = P[(r0 + a) * TP + k];
        ld4<S>(Q + k * TP + c0, *reinterpret_cast<S(*)[4]>(q));
        ld4<S>(Q + k * TP + c0 + 4, q2);
#pragma unroll
        for (int b = 0; b < 4; b++) q[4 + b] = q2[b];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 8; b++) acc[a][b] = fma(p[a], q[b], acc[a][b]);
    }
}

// Factor the upper 32 x 32 tile D (row-major, pitch TP) in place, D = R^T R, and write
// R^-1 (upper) into Di.  One warp.  diag0: the original diagonal of the whole matrix at
// this tile (relative breakdown test d_j > rel_tol * diag0_j).  Returns false on breakdown.
// Lane t keeps column t of the tile in registers.  Step j: lane j's pivot and its reciprocal
// square root were formed at the end of step j - 1, so the step's critical path is one
// broadcast, the scaling of row j, and lane j+1 forming the next pivot from its own values
// (c[j+1] - R(j, j+1)^2); the trailing updates c[i] -= R(j, i) R(j, t) read row j of R through
// shared memory with 16-byte broadcast loads (a shuffle per entry made the 528 broadcasts the
// bulk of the instructions).  FP32: reciprocal square root by the hardware estimate and one
// Newton step (R's diagonal to ~1 ulp).
template <typename S>
__device__ __forceinline__ S chol_rsqrt(S d) {
    if constexpr (sizeof(S) == 4) {
        const float r = rsqrtf(d);
        return r * fmaf(-0.5f * d, r * r, 1.5f);
    } else {
        return 1.0 / sqrt(d);
    }
}
template <typename S>
__device__ __noinline__ bool factor_diag_warp(S *D, S *Di, const S *diag0, S rel_tol) {
    const int lane = threadIdx.x & 31;
    S c[32];
#pragma unroll
    for (int i = 0; i < 32; i++) c[i] = (i <= lane) ? D[i * TP + lane] : S(0);
    const S thr = rel_tol * diag0[lane];                // this lane's column: breakdown threshold
    bool bad = false;
    S own_inv = S(1);                                   // 1 / R(lane, lane)
    // pivot of step 0 (meaningful on lane 0)
    bool okn = (c[0] > S(0)) && isfinite(c[0]) && (c[0] > thr);
    S invn = okn ? chol_rsqrt<S>(c[0]) : S(1);
#pragma unroll
    for (int j = 0; j < 32; j++) {
        const S inv = __shfl_sync(FULL, invn, j);
        const bool ok = __shfl_sync(FULL, okn ? 1 : 0, j) != 0;
        bad |= !ok;
        if (lane == j) {
            if constexpr (sizeof(S) == 4) c[j] = ok ? c[j] * inv : S(1);      // sqrt(d) = d rsqrt(d)
            else c[j] = ok ? sqrt(c[j]) : S(1);
            own_inv = inv;
        } else if (lane > j) {
            c[j] *= inv;                                // lane t now holds R(j, t)
        }
        if (j + 1 < 32) {
            // next pivot, on lane j+1: c[j+1] - R(j, j+1)^2, R(j, j+1) being its own c[j]
            const S pn = c[j + 1] - c[j] * c[j];
            okn = (pn > S(0)) && isfinite(pn) && (pn > thr);
            invn = okn ? chol_rsqrt<S>(pn) : S(1);
        }
        // row j of R to every lane through shared memory (Di is scratch until the inverse is
        // written): one store a lane, then 16-byte broadcast reads
        if (lane > j) Di[lane] = c[j];
        __syncwarp();
        constexpr int VW = 16 / sizeof(S);
#pragma unroll
        for (int q = (j + 1) / VW; q < 32 / VW; q++) {
            S r[VW];
            if constexpr (sizeof(S) == 4) {
                const float4 v = *reinterpret_cast<const float4 *>(Di + q * VW);
                r[0] = v.x; r[1] = v.y; r[2] = v.z; r[3] = v.w;
            } else {
                const double2 v = *reinterpret_cast<const double2 *>(Di + q * VW);
                r[0] = v.x; r[1] = v.y;
            }
#pragma unroll
            for (int e = 0; e < VW; e++) {
                const int i = q * VW + e;
                if (i > j && lane >= i) c[i] -= r[e] * c[j];     // R(j, i) R(j, lane)
            }
        }
        __syncwarp();
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < 32; i++) D[i * TP + lane] = (i <= lane) ? c[i] : S(0);
    __syncwarp();
    // column `lane` of R^-1 by back substitution, R read back from the tile (broadcast
    // reads: every lane reads the same R(i, k)); x[k] = 0 for k > lane
    S x[32];
#pragma unroll
    for (int i = 31; i >= 0; i--) {
        S acc0 = S(0), acc1 = S(0);                     // two chains: half the FMA latency
#pragma unroll
        for (int k = i + 1; k < 32; k += 2) {
            acc0 = fma(D[i * TP + k], x[k], acc0);
            if (k + 1 < 32) acc1 = fma(D[i * TP + k + 1], x[k + 1], acc1);
        }
        const S acc = acc0 + acc1;
        if constexpr (sizeof(S) == 4) {
            const S inv_i = __shfl_sync(FULL, own_inv, i);
            x[i] = (i == lane) ? inv_i : ((i < lane) ? -acc * inv_i : S(0));
        } else {
            const S rii = D[i * TP + i];
            x[i] = (i == lane) ? S(1) / rii : ((i < lane) ? -acc / rii : S(0));
        }
    }
#pragma unroll
    for (int i = 0; i < 32; i++) Di[i * TP + lane] = x[i];
    __syncwarp();
    return !bad;
}

// Store a lane's 4 x 8 block (optionally subtracting from the tile).  FP32: two 16-byte
// accesses per row, lanes of odd row groups taking the upper half (columns c0+4..c0+7) first:
// with the pitch TP = 36 the rows r0 and r0 + 4 lie 16 banks apart, so this order lets every
// 8-lane phase of a 16-byte access cover the 32 banks once (scalar accesses were 8-way
// conflicts and made the trailing update shared-memory bound).
template <typename S>
__device__ __forceinline__ void put_acc(S *T, const S (&acc)[4][8], bool subtract) {
    const int r0 = lane_r0(), c0 = lane_c0();
    if constexpr (sizeof(S) == 4) {
        const bool up = (r0 >> 2) & 1;
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const float4 lo = make_float4(acc[a][0], acc[a][1], acc[a][2], acc[a][3]);
            const float4 hi = make_float4(acc[a][4], acc[a][5], acc[a][6], acc[a][7]);
            float4 *p0 = reinterpret_cast<float4 *>(T + (r0 + a) * TP + c0 + (up ? 4 : 0));
            float4 *p1 = reinterpret_cast<float4 *>(T + (r0 + a) * TP + c0 + (up ? 0 : 4));
            float4 v0 = up ? hi : lo, v1 = up ? lo : hi;
            if (subtract) {
                const float4 o0 = *p0;
                v0 = make_float4(o0.x - v0.x, o0.y - v0.y, o0.z - v0.z, o0.w - v0.w);
            }
            *p0 = v0;
            if (subtract) {
                const float4 o1 = *p1;
                v1 = make_float4(o1.x - v1.x, o1.y - v1.y, o1.z - v1.z, o1.w - v1.w);
            }
            *p1 = v1;
        }
    } else {
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 8; b++) {
                S &t = T[(r0 + a) * TP + c0 + b];
                t = subtract ? t - acc[a][b] : acc[a][b];
            }
    }
}

// Load a 32 x 32 tile of a column-major FP64 matrix into a shared-memory tile (one warp).
// Outside [0, n): identity (so padded diagonal blocks factor trivially).  upper_only:
// entries below the diagonal of the whole matrix read as 0.
template <typename S>
__device__ void load_tile_g(S *T, const double *G, long long ldg, int n, int I, int K, bool upper_only) {
    const int lane = threadIdx.x & 31;
    for (int c = 0; c < TB; c++) {
        const int gi = I * TB + lane, gk = K * TB + c;
        S v;
        if (gi < n && gk < n) v = (!upper_only || gi <= gk) ? (S)G[gi + (long long)gk * ldg] : S(0);
        else v = (gi == gk) ? S(1) : S(0);
        T[lane * TP + c] = v;
    }
}

// Trailing update of step J, G_IK -= R_JI^T R_JK for J < I <= K except tile (J+1, J+1): the
// warps claim tiles from the shared counter *next (set to 1 before the step), so warp 0 joins
// in once it has factored the next diagonal tile.
template <typename S>
__device__ __forceinline__ void trailing_update(S *T, int J, int nt, int *next) {
    const int lane = threadIdx.x & 31, ntiles = nt * (nt + 1) / 2;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(next, 1);
        t = __shfl_sync(FULL, t, 0);
        if (t >= ntiles) break;
        int Ip, Kp;
        untix(t, Ip, Kp);
        const int I = J + 1 + Ip, K = J + 1 + Kp;
        S acc[4][8];
        zero_acc(acc);
        tile_tn<S>(T + (size_t)tix(J, I) * TE, T + (size_t)tix(J, K) * TE, 0, TB, acc);
        put_acc<S>(T + (size_t)tix(I, K) * TE, acc, true);
    }
}

// The J loop of the one-CTA factorisation over tiles resident in shared memory (T: packed
// upper tiles, Dw: scratch tile, diag0: original diagonal).  *bad is set on breakdown.
// Lookahead: while warps 1.. apply step J's trailing update, warp 0 updates the next
// diagonal tile first and factors it, so the one-warp diagonal step (the sequential part)
// overlaps the trailing update instead of following it.
template <typename S>
__device__ void chol_steps(S *T, S *Dw, const S *diag0, int nb, double rel_tol, S *dinv, int *bad) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __shared__ int next_tile;
    if (wid == 0) {
        const bool ok = factor_diag_warp<S>(T, Dw, diag0, (S)rel_tol);
        if (!ok && lane == 0) *bad = 1;
    }
    __syncthreads();
    for (int J = 0; J < nb; J++) {
        if (*bad) break;
        // panel R_JK = R_JJ^-T G_JK (in place; R_JJ^-1 upper: only k <= r contributes)
        for (int K = J + 1 + wid; K < nb; K += nw) {
            S *W = T + (size_t)tix(J, K) * TE;
            S acc[4][8];
            zero_acc(acc);
            tile_tn<S>(Dw, W, 0, lane_r0() + 4, acc);
            __syncwarp();
            put_acc<S>(W, acc, false);
        }
        for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) dinv[(size_t)J * TB * TB + e] = Dw[(e >> 5) * TP + (e & 31)];
        if (threadIdx.x == 0) next_tile = 1;
        __syncthreads();
        // trailing update G_IK -= R_JI^T R_JK, J < I <= K: tile (J+1, J+1) (t = 0) and the
        // next diagonal factorisation on warp 0, the other tiles on whichever warp is free
        const int nt = nb - J - 1;
        if (nt > 0) {
            if (wid == 0) {
                S acc[4][8];
                zero_acc(acc);
                tile_tn<S>(T + (size_t)tix(J, J + 1) * TE, T + (size_t)tix(J, J + 1) * TE, 0, TB, acc);
                put_acc<S>(T + (size_t)tix(J + 1, J + 1) * TE, acc, true);
                __syncwarp();
                const bool ok = factor_diag_warp<S>(T + (size_t)tix(J + 1, J + 1) * TE, Dw, diag0 + (J + 1) * TB,
                                                    (S)rel_tol);
                if (!ok && lane == 0) *bad = 1;
            }
            trailing_update<S>(T, J, nt, &next_tile);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- one CTA, all tiles in smem
// Shared memory: nb(nb+1)/2 tiles + 1 scratch tile (diagonal inverse) + nb*32 diagonal.
// Outputs: R in G (upper, zero below), the inverted diagonal tiles in dinv (nb row-major
// 32 x 32 tiles, compute type).
template <typename S>
constexpr int chol_smem_threads() { return 256; }   // the register factorisation needs > 128 per thread

template <typename S>
__global__ void __launch_bounds__(chol_smem_threads<S>()) chol_smem_kernel(double *G, long long ldg, int n, int nb, double rel_tol,
                                                        S *dinv, int *flag) {
    extern __shared__ __align__(16) unsigned char shraw[];
    S *T = (S *)shraw;
    const int ntile = tix(0, nb);
    S *Dw = T + (size_t)ntile * TE;
    S *diag0 = Dw + TE;
    __shared__ int bad;
    const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int t = wid; t < ntile; t += nw) {
        int I, K;
        untix(t, I, K);
        load_tile_g<S>(T + (size_t)t * TE, G, ldg, n, I, K, true);
    }
    for (int j = threadIdx.x; j < nb * TB; j += blockDim.x) diag0[j] = (j < n) ? (S)G[j + (long long)j * ldg] : S(1);
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    chol_steps<S>(T, Dw, diag0, nb, rel_tol, dinv, &bad);
    if (bad) {
        if (threadIdx.x == 0) atomicExch(flag, 1);
        return;
    }
    // R -> G (column-major, zero below the diagonal)
    for (long long e = threadIdx.x; e < (long long)n * n; e += blockDim.x) {
        const int k = (int)(e / n), i = (int)(e - (long long)k * n);
        double v = 0.0;
        if (i <= k) v = (double)T[(size_t)tix(i >> 5, k >> 5) * TE + (i & 31) * TP + (k & 31)];
        G[i + (long long)k * ldg] = v;
    }
}

// ---------------------------------------------------------------- FP32, packed tiles in/out
// Gt: the Gram as FP32 packed upper tiles (32 x 32 row-major, pitch 32, padded with the
// identity; written by gram_tiles_f32).  All tiles come into shared memory by 16-byte
// asynchronous copies; on return Gt holds R in the same layout (zero below the diagonal
// of the diagonal tiles).  Rout (optional): R as FP64, column-major, zero below.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

constexpr int CHOL_F32_THREADS = 512;
__global__ void __launch_bounds__(CHOL_F32_THREADS) chol_tiles_f32_kernel(float *Gt, int n, int nb, double rel_tol,
                                                                          float *dinv, int *flag) {
    extern __shared__ __align__(16) unsigned char shraw[];
    float *T = (float *)shraw;
    const int ntile = tix(0, nb);
    float *Dw = T + (size_t)ntile * TE;
    float *diag0 = Dw + TE;
    __shared__ int bad;
    const int nchunk = ntile * TB * 8;                     // 16-byte chunks: 8 per tile row
    for (int e = threadIdx.x; e < nchunk; e += blockDim.x) {
        const int t = e >> 8, r = (e >> 3) & 31, q = e & 7;
        cp_async16(T + (size_t)t * TE + r * TP + q * 4, Gt + (size_t)t * TB * TB + r * TB + q * 4);
    }
    cp_async_wait_all();
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int j = threadIdx.x; j < nb * TB; j += blockDim.x) {
        const int J = j >> 5, jj = j & 31;
        diag0[j] = T[(size_t)tix(J, J) * TE + jj * TP + jj];
    }
    __syncthreads();
    chol_steps<float>(T, Dw, diag0, nb, rel_tol, dinv, &bad);
    if (bad) {
        if (threadIdx.x == 0) atomicExch(flag, 1);
        return;
    }
    // R tiles back to Gt (16-byte stores)
    for (int e = threadIdx.x; e < nchunk; e += blockDim.x) {
        const int t = e >> 8, r = (e >> 3) & 31, q = e & 7;
        *reinterpret_cast<float4 *>(Gt + (size_t)t * TB * TB + r * TB + q * 4) =
            *reinterpret_cast<const float4 *>(T + (size_t)t * TE + r * TP + q * 4);
    }
}

// R as FP64, column-major, zero below, from the packed FP32 tiles: a separate grid-wide pass,
// because FP64 conversions from one SM (FP64 units are few on GB300) cost ~20 us at n = 272.
__global__ void tiles_to_fp64_kernel(const float *Gt, int n, double *R, long long ldr) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)n * n;
         e += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(e / n), i = (int)(e - (long long)k * n);
        R[i + (long long)k * ldr] =
            (i <= k) ? (double)Gt[(size_t)tix(i >> 5, k >> 5) * TB * TB + (i & 31) * TB + (k & 31)] : 0.0;
    }
}

// ---------------------------------------------------------------- tiles in global memory
// Working storage: packed upper tiles, each 32 x 32 row-major (pitch 32), compute type.
template <typename S>
__global__ void chol_gload_kernel(const double *G, long long ldg, int n, int nb, S *Wt, S *diag0) {
    const long long tot = (long long)tix(0, nb) * TB * TB;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
        const int t = (int)(e >> 10), w = (int)(e & 1023), r = w >> 5, c = w & 31;
        int I, K;
        untix(t, I, K);
        const int gi = I * TB + r, gk = K * TB + c;
        S v;
        if (gi < n && gk < n) v = (gi <= gk) ? (S)G[gi + (long long)gk * ldg] : S(0);
        else v = (gi == gk) ? S(1) : S(0);
        Wt[e] = v;
        if (I == K && r == c) diag0[gi] = (gi < n) ? (S)G[gi + (long long)gi * ldg] : S(1);
    }
}

template <typename S>
__device__ __forceinline__ void gtile_to_smem(S *T, const S *g) {
    const int lane = threadIdx.x & 31;
    for (int r = 0; r < TB; r++) T[r * TP + lane] = g[r * TB + lane];
}
template <typename S>
__device__ __forceinline__ void acc_to_gtile(S *g, const S (&acc)[4][8], bool subtract) {
    const int r0 = lane_r0(), c0 = lane_c0();
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 8; b++) {
            S &t = g[(r0 + a) * TB + c0 + b];
            t = subtract ? t - acc[a][b] : acc[a][b];
        }
}

// Step J, panel: CTA b (one warp) factors the diagonal tile itself (all CTAs agree) and
// forms R_JK, K = J + b.  CTA 0 writes R_JJ to Rd (not over the tile the other CTAs are
// reading) and its inverse to dinv.
template <typename S>
__global__ void __launch_bounds__(32) chol_gpanel_kernel(S *Wt, int nb, int J, const S *diag0, double rel_tol,
                                                         S *dinv, S *Rd, int *flag) {
    __shared__ __align__(16) S D[TE], Di[TE], W[TE];
    const int K = J + blockIdx.x;
    gtile_to_smem<S>(D, Wt + (size_t)tix(J, J) * TB * TB);
    __syncwarp();
    const bool ok = factor_diag_warp<S>(D, Di, diag0 + J * TB, (S)rel_tol);
    if (!ok) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(flag, 1);
        return;
    }
    const int lane = threadIdx.x;
    if (K == J) {
        for (int r = 0; r < TB; r++) {
            Rd[(size_t)J * TB * TB + r * TB + lane] = D[r * TP + lane];
            dinv[(size_t)J * TB * TB + r * TB + lane] = Di[r * TP + lane];
        }
        return;
    }
    S *g = Wt + (size_t)tix(J, K) * TB * TB;
    gtile_to_smem<S>(W, g);
    __syncwarp();
    S acc[4][8];
    zero_acc(acc);
    tile_tn<S>(Di, W, 0, lane_r0() + 4, acc);
    acc_to_gtile<S>(g, acc, false);
}

// Step J, trailing update: CTA t (one warp) updates tile (I, K), J < I <= K.
template <typename S>
__global__ void __launch_bounds__(32) chol_gupdate_kernel(S *Wt, int nb, int J) {
    __shared__ __align__(16) S P[TE], Q[TE];
    int Ip, Kp;
    untix(blockIdx.x, Ip, Kp);
    const int I = J + 1 + Ip, K = J + 1 + Kp;
    gtile_to_smem<S>(P, Wt + (size_t)tix(J, I) * TB * TB);
    gtile_to_smem<S>(Q, Wt + (size_t)tix(J, K) * TB * TB);
    __syncwarp();
    S acc[4][8];
    zero_acc(acc);
    tile_tn<S>(P, Q, 0, TB, acc);
    acc_to_gtile<S>(Wt + (size_t)tix(I, K) * TB * TB, acc, true);
}

template <typename S>
__global__ void chol_gstore_kernel(const S *Wt, const S *Rd, int n, double *G, long long ldg) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)n * n;
         e += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(e / n), i = (int)(e - (long long)k * n);
        double v = 0.0;
        const int I = i >> 5, K = k >> 5;
        if (i <= k) v = (double)((I == K) ? Rd[(size_t)I * TB * TB + (i & 31) * TB + (k & 31)]
                                          : Wt[(size_t)tix(I, K) * TB * TB + (i & 31) * TB + (k & 31)]);
        G[i + (long long)k * ldg] = v;
    }
}

// ---------------------------------------------------------------- triangular inverse
// CTA J computes block column J of X = R^-1 (R: FP64, column-major, upper).  Warps split
// the K-sum of each row block I, accumulate into a shared tile, and warp 0 applies
// -R_II^-1.  X_KJ for K > I are read back from X (written earlier by this CTA).
template <typename S, typename To>
__global__ void __launch_bounds__(512) tri_inv_tiles_kernel(const double *R, long long ldr, int n, int nb,
                                                            const S *dinv, To *X, long long ldx) {
    extern __shared__ __align__(16) unsigned char shraw[];
    const int J = blockIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    S *Acc = (S *)shraw;                  // the K-sum
    S *Dt = Acc + TE;                     // R_II^-1
    S *Pw = Dt + TE + (size_t)wid * 2 * TE, *Qw = Pw + TE;   // per-warp R_IK, X_KJ
    const int jw = min(TB, n - J * TB);
    // X_JJ = R_JJ^-1; below the diagonal of the block column: zero
    for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
        const int r = e & 31, c = e >> 5;
        const int gi = J * TB + r, gk = J * TB + c;
        if (gi < n && gk < n) X[gi + (long long)gk * ldx] = (To)((r <= c) ? dinv[(size_t)J * TB * TB + r * TB + c] : S(0));
    }
    for (long long e = threadIdx.x; e < (long long)jw * n; e += blockDim.x) {
        const int c = (int)(e / n), gi = (int)(e - (long long)c * n);
        if (gi >= (J + 1) * TB) X[gi + (long long)(J * TB + c) * ldx] = (To)0;
    }
    for (int e = threadIdx.x; e < TE; e += blockDim.x) Acc[e] = S(0);
    __syncthreads();
    for (int I = J - 1; I >= 0; I--) {
        // partial sums over K = I+1 .. J, one tile product per warp at a time
        S acc[4][8];
        zero_acc(acc);
        bool any = false;
        for (int K = I + 1 + wid; K <= J; K += nw) {
            any = true;
            for (int c = 0; c < TB; c++) {
                const int gi = I * TB + lane, gk = K * TB + c;                 // R_IK (row lane, col c)
                Pw[lane * TP + c] = (gi < n && gk < n) ? (S)R[gi + (long long)gk * ldr] : S(0);
                const int xi = K * TB + lane, xk = J * TB + c;                 // X_KJ
                Qw[lane * TP + c] = (xi < n && xk < n) ? (S)X[xi + (long long)xk * ldx] : S(0);
            }
            __syncwarp();
            tile_nn<S>(Pw, Qw, 0, TB, acc);
            __syncwarp();
        }
        if (any) {
            const int r0 = lane_r0(), c0 = lane_c0();
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 8; b++) atomicAdd(&Acc[(r0 + a) * TP + c0 + b], acc[a][b]);
        }
        for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) Dt[(e >> 5) * TP + (e & 31)] = dinv[(size_t)I * TB * TB + e];
        __syncthreads();
        if (wid == 0) {
            S o[4][8];
            zero_acc(o);
            tile_nn<S>(Dt, Acc, 0, TB, o);
            const int r0 = lane_r0(), c0 = lane_c0();
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 8; b++) {
                    const int gi = I * TB + r0 + a, gk = J * TB + c0 + b;
                    if (gi < n && gk < n) X[gi + (long long)gk * ldx] = (To)(-o[a][b]);
                }
        }
        __syncthreads();
        for (int e = threadIdx.x; e < TE; e += blockDim.x) Acc[e] = S(0);
        __syncthreads();
    }
}

// ---------------------------------------------------------------- C = A B, A and B upper
// CTA t: tile (I, K) of C (upper tiles first, then the strictly lower tiles, which are
// zeroed).  256 threads stage A_IL and B_LK; warp 0 accumulates the products.
template <typename S>
__global__ void __launch_bounds__(256) tri_mul_upper_kernel(const double *A, long long lda, const double *B,
                                                            long long ldb, double *C, long long ldc, int n, int nb) {
    __shared__ __align__(16) S P[TE], Q[TE];
    const int t = blockIdx.x;
    const int ntile = tix(0, nb);
    int I, K;
    if (t >= ntile) {
        int Kp, Ip;
        untix(t - ntile, Kp, Ip);                      // Kp <= Ip
        I = Ip + 1;
        K = Kp;
        for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
            const int gi = I * TB + (e & 31), gk = K * TB + (e >> 5);
            if (gi < n && gk < n) C[gi + (long long)gk * ldc] = 0.0;
        }
        return;
    }
    untix(t, I, K);
    S acc[4][8];
    zero_acc(acc);
    for (int L = I; L <= K; L++) {
        for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
            const int r = e & 31, c = e >> 5;
            const int gi = I * TB + r, gl = L * TB + c;
            P[r * TP + c] = (gi < n && gl < n && gi <= gl) ? (S)A[gi + (long long)gl * lda] : S(0);
            const int bi = L * TB + r, bk = K * TB + c;
            Q[r * TP + c] = (bi < n && bk < n && bi <= bk) ? (S)B[bi + (long long)bk * ldb] : S(0);
        }
        __syncthreads();
        if (threadIdx.x < 32) tile_nn<S>(P, Q, 0, TB, acc);
        __syncthreads();
    }
    if (threadIdx.x < 32) {
        const int r0 = lane_r0(), c0 = lane_c0();
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 8; b++) {
                const int gi = I * TB + r0 + a, gk = K * TB + c0 + b;
                if (gi < n && gk < n) C[gi + (long long)gk * ldc] = (gi <= gk) ? (double)acc[a][b] : 0.0;
            }
    }
}

// ---------------------------------------------------------------- Q = Y R^-1 by slabs
// One CTA per slab of BM rows of Y (m x n): block column J of Q is
//   Q_J = (Y_J - Q_{:, 0:J} R_{0:J, J}) R_JJ^-1,
// with the slab's finished columns of Q kept in shared memory (column-major, pitch BM + 4,
// so a thread's RPT rows are one 16-byte load) and R's block column J staged per step
// (R_JJ^-1 from the factorisation's inverted diagonal tiles).  Thread t: rows
// (t / 8) * RPT .. + RPT - 1 of the slab, columns (t % 8) * 4 .. + 3 of the block.
constexpr int TRSM_THREADS = 256;
// R comes either as FP64 column-major (R, ldr) or, when Rt is given, as packed upper
// tiles in the compute type (the layout chol_tiles_f32_kernel leaves), staged by 16-byte
// asynchronous copies.
template <typename T, typename S, int BM>
__global__ void __launch_bounds__(TRSM_THREADS) trsm_slab_kernel(const T *Y, long long ldy, const double *R,
                                                                 long long ldr, const S *Rt, const S *dinv, T *Q,
                                                                 long long ldq, long long m, int n, int nb) {
    constexpr int RPT = BM / 32;
    static_assert(RPT == 4, "one 16-byte row group per thread");
    constexpr int BP = BM + 4;                        // column pitch of the slab
    extern __shared__ __align__(16) unsigned char shraw[];
    S *Qs = (S *)shraw;                               // (nb * 32) columns x BP
    S *Rc = Qs + (size_t)nb * TB * BP;                // (nb * 32) x TP: block column J of R
    S *Dv = Rc + (size_t)nb * TB * TP;                // 32 x TP: R_JJ^-1
    const long long row0 = (long long)blockIdx.x * BM;
    const int t = threadIdx.x;
    const int rg = (t >> 3) * RPT, cg = (t & 7) * 4;
    for (int J = 0; J < nb; J++) {
        const int kr = J * TB;                        // rows of R above the diagonal tile
        if constexpr (sizeof(S) == 4) {
            if (Rt) {
                constexpr int CPR = TB * sizeof(S) / 16;      // 16-byte chunks per tile row
                for (int e = t; e < kr * CPR; e += TRSM_THREADS) {
                    const int I = e / (TB * CPR), r = (e / CPR) % TB, q = e % CPR;
                    cp_async16(Rc + (I * TB + r) * TP + q * 4, Rt + (size_t)tix(I, J) * TB * TB + r * TB + q * 4);
                }
                for (int e = t; e < TB * CPR; e += TRSM_THREADS) {
                    const int r = e / CPR, q = e % CPR;
                    cp_async16(Dv + r * TP + q * 4, dinv + (size_t)J * TB * TB + r * TB + q * 4);
                }
                cp_async_wait_all();
            }
        }
        if (!Rt) {
            for (int e = t; e < kr * TB; e += TRSM_THREADS) {
                const int k = e % kr, c = e / kr;
                const int gc = kr + c;
                Rc[k * TP + c] = (gc < n) ? (S)R[k + (long long)gc * ldr] : S(0);
            }
            for (int e = t; e < TB * TB; e += TRSM_THREADS) Dv[(e >> 5) * TP + (e & 31)] = dinv[(size_t)J * TB * TB + e];
        }
        S acc[RPT][4];
#pragma unroll
        for (int a = 0; a < RPT; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) {
                const long long gr = row0 + rg + a;
                const int gc = kr + cg + b;
                acc[a][b] = (gr < m && gc < n) ? (S)Y[gr + (long long)gc * ldy] : S(0);
            }
        __syncthreads();
        for (int k = 0; k < kr; k++) {
            S r4[4], q[RPT];
            ld4<S>(Rc + k * TP + cg, r4);
            ld4<S>(Qs + (size_t)k * BP + rg, q);
#pragma unroll
            for (int a = 0; a < RPT; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = fma(-q[a], r4[b], acc[a][b]);
        }
        // the diagonal block: Q_J = T R_JJ^-1 (T staged through the slab's column block J)
#pragma unroll
        for (int a = 0; a < RPT; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) Qs[(size_t)(kr + cg + b) * BP + rg + a] = acc[a][b];
        __syncthreads();
        S o[RPT][4];
#pragma unroll
        for (int a = 0; a < RPT; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) o[a][b] = S(0);
#pragma unroll 4
        for (int k = 0; k < TB; k++) {
            S d4[4], q[RPT];
            ld4<S>(Dv + k * TP + cg, d4);
            ld4<S>(Qs + (size_t)(kr + k) * BP + rg, q);
#pragma unroll
            for (int a = 0; a < RPT; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) o[a][b] = fma(q[a], d4[b], o[a][b]);
        }
        __syncthreads();
#pragma unroll
        for (int a = 0; a < RPT; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) {
                Qs[(size_t)(kr + cg + b) * BP + rg + a] = o[a][b];
                const long long gr = row0 + rg + a;
                const int gc = kr + cg + b;
                if (gr < m && gc < n) Q[gr + (long long)gc * ldq] = (T)o[a][b];
            }
        __syncthreads();
    }
}

template <typename S>
constexpr int smem_nb_max() { return sizeof(S) == 4 ? 9 : 6; }

// FP32 slab solve Q R = Y on the tensor cores (mma.sync m16n8k8, 3xTF32: hi x hi + hi x lo +
// lo x hi, each operand split into a TF32 high part and the TF32 rounding of the remainder,
// so products carry ~FP32 accuracy).  One CTA per 128-row slab, warp w owns rows
// [16 w, 16 w + 16) of it.  Block column J: P = Q_{<J} R_{<J,J} (A fragments from the warp's
// rows of the slab's Q, kept in shared memory row-major, pitch QP; B fragments from R's block
// column J, staged once per J for all warps), T = Y_J - P, then Q_J = T R_JJ^-1 (T staged
// through the warp's own rows of the slab).  Only the staging of R's block column needs block
// barriers; a warp's rows depend on nothing but its own earlier columns.  R comes as the packed
// FP32 upper tiles chol_tiles_f32_kernel leaves, R_JJ^-1 from its dinv (identity-padded
// beyond n, so padded columns solve to zero).  Shared memory: 128 x QP (Q) + 256 x RPB (R block
// column) + 32 x RPB (R_JJ^-1) floats; the pitches make every fragment load conflict-free
// (QP = 4 mod 32 for A, RPB = 8 mod 32 for B).
__device__ __forceinline__ uint32_t tf32_hi(float x) {
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
    return h;
}
__device__ __forceinline__ void tf32_split(float x, uint32_t &h, uint32_t &l) {
    h = tf32_hi(x);
    l = tf32_hi(x - __uint_as_float(h));
}
__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
// acc (16 x 32: four 16 x 8 tiles) += A (the warp's 16 rows, columns [k0, k1) of As, pitch ap)
//                                     x B (rows [k0, k1) of Bs, 32 columns, pitch bp)
__device__ __forceinline__ void mma3_rows(float (&acc)[4][4], const float *As, int ap, const float *Bs, int bp, int k0,
                                          int k1) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    for (int k = k0; k < k1; k += 8) {
        uint32_t ah[4], al[4];
        tf32_split(As[g * ap + k + t], ah[0], al[0]);
        tf32_split(As[(g + 8) * ap + k + t], ah[1], al[1]);
        tf32_split(As[g * ap + k + t + 4], ah[2], al[2]);
        tf32_split(As[(g + 8) * ap + k + t + 4], ah[3], al[3]);
#pragma unroll
        for (int nt = 0; nt < 4; nt++) {
            uint32_t bh0, bl0, bh1, bl1;
            tf32_split(Bs[(k + t) * bp + nt * 8 + g], bh0, bl0);
            tf32_split(Bs[(k + t + 4) * bp + nt * 8 + g], bh1, bl1);
            mma_tf32(acc[nt], al, bh0, bh1);
            mma_tf32(acc[nt], ah, bl0, bl1);
            mma_tf32(acc[nt], ah, bh0, bh1);
        }
    }
}
constexpr int TRSM_MMA_BM = 128, RPB = 40;
__global__ void __launch_bounds__(256) trsm_mma_kernel(const float *Y, long long ldy, const float *Rt, const float *dinv,
                                                      float *Q, long long ldq, long long m, int n, int nb) {
    extern __shared__ __align__(16) unsigned char shraw[];
    const int QP = nb * TB + 4;                       // row pitch of the slab's Q (conflict-free fragments)
    float *Qs = (float *)shraw;                       // 128 x QP
    float *Rc = Qs + (size_t)TRSM_MMA_BM * QP;        // (nb - 1) * 32 x RPB: rows [0, 32 J) of block column J
    float *Dv = Rc + (size_t)(nb - 1) * TB * RPB;     // 32 x RPB: R_JJ^-1
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
    const long long row0 = (long long)blockIdx.x * TRSM_MMA_BM + wid * 16;
    float *Qw = Qs + (size_t)wid * 16 * QP;           // this warp's 16 rows
    constexpr int CPR = TB / 4;                       // 16-byte chunks per tile row
    for (int J = 0; J < nb; J++) {
        const int kr = J * TB;
        __syncthreads();                              // every warp is done with the previous R block column
        for (int e = threadIdx.x; e < kr * CPR; e += blockDim.x) {
            const int I = e / (TB * CPR), r = (e / CPR) % TB, q = e % CPR;
            cp_async16(Rc + (I * TB + r) * RPB + q * 4, Rt + (size_t)tix(I, J) * TB * TB + r * TB + q * 4);
        }
        for (int e = threadIdx.x; e < TB * CPR; e += blockDim.x) {
            const int r = e / CPR, q = e % CPR;
            cp_async16(Dv + r * RPB + q * 4, dinv + (size_t)J * TB * TB + r * TB + q * 4);
        }
        cp_async_wait_all();
        __syncthreads();
        float acc[4][4];
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[nt][e] = 0.f;
        if (kr > 0) mma3_rows(acc, Qw, QP, Rc, RPB, 0, kr);
        // T = Y_J - P, staged into the warp's rows of column block J
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int r = g + (e >> 1) * 8, c = nt * 8 + 2 * t + (e & 1);
                const long long gr = row0 + r;
                const int gc = kr + c;
                const float y = (gr < m && gc < n) ? Y[gr + (long long)gc * ldy] : 0.f;
                Qw[r * QP + kr + c] = y - acc[nt][e];
            }
        __syncwarp();
        float o[4][4];
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int e = 0; e < 4; e++) o[nt][e] = 0.f;
        mma3_rows(o, Qw + kr, QP, Dv, RPB, 0, TB);
        __syncwarp();
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int r = g + (e >> 1) * 8, c = nt * 8 + 2 * t + (e & 1);
                Qw[r * QP + kr + c] = o[nt][e];
                const long long gr = row0 + r;
                const int gc = kr + c;
                if (gr < m && gc < n) Q[gr + (long long)gc * ldq] = o[nt][e];
            }
        __syncwarp();
    }
}

// C (M x N) = A (M x K) B (K x N), FP32, all column-major, on the tensor cores in 3xTF32
// (mma.sync m16n8k8): the factor formation U = Q Vk, V = Qh Uk of the mixed modes (K = l),
// kept at FP32 accuracy without the CUDA-core rate.  CTA tile 128 x 64, K in chunks of 32,
// both operands split once per chunk into TF32 high and low parts in shared memory (A as
// [row][k] with pitch 36 and B as [k][col] with pitch 72: conflict-free fragment loads); the
// next chunk's global loads are issued before the current chunk's products.  8 warps in a
// 4 x 2 grid of 32 x 32 warp tiles.
constexpr int G3_BM = 128, G3_BN = 64, G3_BK = 32, G3_AP = G3_BK + 4, G3_BP = G3_BN + 8;
__global__ void __launch_bounds__(256) gemm_nn_3xtf32_kernel(const float *A, long long lda, const float *B,
                                                            long long ldb, float *C, long long ldc, int M, int N,
                                                            int K) {
    extern __shared__ __align__(16) unsigned char shraw[];
    uint32_t *Ah = (uint32_t *)shraw, *Al = Ah + G3_BM * G3_AP;
    uint32_t *Bh = Al + G3_BM * G3_AP, *Bl = Bh + G3_BK * G3_BP;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, g = lane >> 2, t = lane & 3;
    const long long row0 = (long long)blockIdx.x * G3_BM;
    const int col0 = blockIdx.y * G3_BN;
    const int wm = (wid & 3) * 32, wn = (wid >> 2) * 32;
    // global -> register mapping: A rows tid % 128, k = tid / 128 + 2 i; B k = tid % 32, cols tid / 32 + 8 i
    const int ar = tid & 127, ak = tid >> 7, bk = tid & 31, bc = tid >> 5;
    const bool arow_ok = row0 + ar < M;
    float ra[16], rb[8];
    auto load = [&](int k0) {
#pragma unroll
        for (int i = 0; i < 16; i++) {
            const int k = k0 + ak + 2 * i;
            ra[i] = (arow_ok && k < K) ? A[row0 + ar + (long long)k * lda] : 0.f;
        }
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int c = col0 + bc + 8 * i, k = k0 + bk;
            rb[i] = (c < N && k < K) ? B[k + (long long)c * ldb] : 0.f;
        }
    };
    float acc[2][4][4];
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 4; b++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[a][b][e] = 0.f;
    load(0);
    for (int k0 = 0; k0 < K; k0 += G3_BK) {
        __syncthreads();                                  // the previous chunk's fragments are read
#pragma unroll
        for (int i = 0; i < 16; i++) {
            uint32_t h, l;
            tf32_split(ra[i], h, l);
            Ah[ar * G3_AP + ak + 2 * i] = h;
            Al[ar * G3_AP + ak + 2 * i] = l;
        }
#pragma unroll
        for (int i = 0; i < 8; i++) {
            uint32_t h, l;
            tf32_split(rb[i], h, l);
            Bh[bk * G3_BP + bc + 8 * i] = h;
            Bl[bk * G3_BP + bc + 8 * i] = l;
        }
        __syncthreads();
        if (k0 + G3_BK < K) load(k0 + G3_BK);
#pragma unroll
        for (int kk = 0; kk < G3_BK; kk += 8) {
            uint32_t ah[2][4], al[2][4], bh[4][2], bl[4][2];
#pragma unroll
            for (int a = 0; a < 2; a++) {
                const int r = wm + a * 16 + g;
                ah[a][0] = Ah[r * G3_AP + kk + t];           al[a][0] = Al[r * G3_AP + kk + t];
                ah[a][1] = Ah[(r + 8) * G3_AP + kk + t];     al[a][1] = Al[(r + 8) * G3_AP + kk + t];
                ah[a][2] = Ah[r * G3_AP + kk + t + 4];       al[a][2] = Al[r * G3_AP + kk + t + 4];
                ah[a][3] = Ah[(r + 8) * G3_AP + kk + t + 4]; al[a][3] = Al[(r + 8) * G3_AP + kk + t + 4];
            }
#pragma unroll
            for (int b = 0; b < 4; b++) {
                const int c = wn + b * 8 + g;
                bh[b][0] = Bh[(kk + t) * G3_BP + c];     bl[b][0] = Bl[(kk + t) * G3_BP + c];
                bh[b][1] = Bh[(kk + t + 4) * G3_BP + c]; bl[b][1] = Bl[(kk + t + 4) * G3_BP + c];
            }
#pragma unroll
            for (int a = 0; a < 2; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    mma_tf32(acc[a][b], al[a], bh[b][0], bh[b][1]);
                    mma_tf32(acc[a][b], ah[a], bl[b][0], bl[b][1]);
                    mma_tf32(acc[a][b], ah[a], bh[b][0], bh[b][1]);
                }
        }
    }
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 4; b++)
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const long long r = row0 + wm + a * 16 + g + (e >> 1) * 8;
                const int c = col0 + wn + b * 8 + 2 * t + (e & 1);
                if (r < M && c < N) C[r + (long long)c * ldc] = acc[a][b][e];
            }
}

// ---------------------------------------------------------------- Cholesky and slab solve fused
// One cooperative launch of 1 + ceil(m / 128) CTAs (all co-resident): CTA 0 runs the one-CTA
// tiled Cholesky of chol_tiles_f32_kernel on the packed Gram and publishes block row J of R (and
// R_JJ^-1) to global memory as soon as step J's panel is done, then releases ready[J]; the other
// CTAs run the 3xTF32 slab solve of trsm_mma_kernel, waiting on ready[J] (acquire) before block
// column J -- which is complete once rows 0..J are published.  The solve of block column J thus
// runs while the Cholesky factors block J + 1 instead of after the whole factorisation.  Waits
// are bounded (~1 s of SM cycles, then FLAG_TIMEOUT and return); a breakdown releases every
// flag as -1 and the slabs return (the caller falls back to Householder QR as before).
__device__ __forceinline__ int ld_acquire_gpu(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(int *p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// chol_steps with the per-step publication (FP32, tiles in shared memory).  Block row J is
// published by warps 1.. (copy to Gt with R_JJ^-1 to dinv, fence, a named barrier among them,
// then the release of ready[J]) while warp 0 already updates and factors diagonal tile J + 1:
// the publication stays off the sequential chain of diagonal steps.
__device__ void chol_steps_publish(float *T, float *Dw, const float *diag0, int nb, double rel_tol, float *dinv,
                                   int *bad, float *Gt, int *ready) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int npub = (int)blockDim.x - 32;            // publishing threads (warps 1..)
    __shared__ int next_tile;
    if (wid == 0) {
        const bool ok = factor_diag_warp<float>(T, Dw, diag0, (float)rel_tol);
        if (!ok && lane == 0) *bad = 1;
    }
    __syncthreads();
    for (int J = 0; J < nb; J++) {
        if (*bad) return;
        for (int K = J + 1 + wid; K < nb; K += nw) {
            float *W = T + (size_t)tix(J, K) * TE;
            float acc[4][8];
            zero_acc(acc);
            tile_tn<float>(Dw, W, 0, lane_r0() + 4, acc);
            __syncwarp();
            put_acc<float>(W, acc, false);
        }
        // R_JJ^-1 leaves Dw before warp 0 overwrites it with step J + 1's inverse
        if (wid > 0)
            for (int e = threadIdx.x - 32; e < TB * TB; e += npub) dinv[(size_t)J * TB * TB + e] = Dw[(e >> 5) * TP + (e & 31)];
        if (threadIdx.x == 0) next_tile = 1;
        __syncthreads();
        const int nt = nb - J - 1;
        if (wid == 0) {
            if (nt > 0) {
                float acc[4][8];
                zero_acc(acc);
                tile_tn<float>(T + (size_t)tix(J, J + 1) * TE, T + (size_t)tix(J, J + 1) * TE, 0, TB, acc);
                put_acc<float>(T + (size_t)tix(J + 1, J + 1) * TE, acc, true);
                __syncwarp();
                const bool ok = factor_diag_warp<float>(T + (size_t)tix(J + 1, J + 1) * TE, Dw, diag0 + (J + 1) * TB,
                                                        (float)rel_tol);
                if (!ok && lane == 0) *bad = 1;
            }
        } else {
            // block row J of R is final: publish it
            for (int e = threadIdx.x - 32; e < (nb - J) * TB * TB; e += npub) {
                const int K = J + e / (TB * TB), w = e % (TB * TB);
                Gt[(size_t)tix(J, K) * TB * TB + w] = T[(size_t)tix(J, K) * TE + (w >> 5) * TP + (w & 31)];
            }
            __threadfence();
            asm volatile("bar.sync 1, %0;" ::"r"(npub) : "memory");
            if (threadIdx.x == 32) st_release_gpu(ready + J, 1);
        }
        if (nt > 0) trailing_update<float>(T, J, nt, &next_tile);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256, 1) chol_trsm_fused_kernel(float *Gt, int n, int nb, double rel_tol, float *dinv,
                                                                int *flags, int *ready, const float *Y, long long ldy,
                                                                float *Q, long long ldq, long long m) {
    extern __shared__ __align__(16) unsigned char shraw[];
    __shared__ int bad, go;
    if (blockIdx.x == 0) {
        float *T = (float *)shraw;
        const int ntile = tix(0, nb);
        float *Dw = T + (size_t)ntile * TE;
        float *diag0 = Dw + TE;
        const int nchunk = ntile * TB * 8;
        for (int e = threadIdx.x; e < nchunk; e += blockDim.x) {
            const int t = e >> 8, r = (e >> 3) & 31, q = e & 7;
            cp_async16(T + (size_t)t * TE + r * TP + q * 4, Gt + (size_t)t * TB * TB + r * TB + q * 4);
        }
        cp_async_wait_all();
        if (threadIdx.x == 0) bad = 0;
        __syncthreads();
        for (int j = threadIdx.x; j < nb * TB; j += blockDim.x) {
            const int J = j >> 5, jj = j & 31;
            diag0[j] = T[(size_t)tix(J, J) * TE + jj * TP + jj];
        }
        __syncthreads();
        chol_steps_publish(T, Dw, diag0, nb, rel_tol, dinv, &bad, Gt, ready);
        __syncthreads();
        if (bad && threadIdx.x == 0) {
            atomicExch(flags + FLAG_CHOL_BREAKDOWN, 1);
            __threadfence();
            for (int J = 0; J < nb; J++) st_release_gpu(ready + J, -1);
        }
        return;
    }
    // ---- slab (blockIdx.x - 1): trsm_mma_kernel with a wait before each block column
    const int QP = nb * TB + 4;
    float *Qs = (float *)shraw;
    float *Rc = Qs + (size_t)TRSM_MMA_BM * QP;
    float *Dv = Rc + (size_t)(nb - 1) * TB * RPB;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
    const long long row0 = (long long)(blockIdx.x - 1) * TRSM_MMA_BM + wid * 16;
    float *Qw = Qs + (size_t)wid * 16 * QP;
    constexpr int CPR = TB / 4;
    for (int J = 0; J < nb; J++) {
        const int kr = J * TB;
        __syncthreads();
        if (threadIdx.x == 0) {
            const long long t0 = clock64();
            int v;
            while ((v = ld_acquire_gpu(ready + J)) == 0) {
                if (clock64() - t0 > (1ll << 31)) {
                    atomicExch(flags + FLAG_TIMEOUT, 1);
                    v = -1;
                    break;
                }
                __nanosleep(200);
            }
            go = v;
        }
        __syncthreads();
        if (go < 0) return;
        for (int e = threadIdx.x; e < kr * CPR; e += blockDim.x) {
            const int I = e / (TB * CPR), r = (e / CPR) % TB, q = e % CPR;
            cp_async16(Rc + (I * TB + r) * RPB + q * 4, Gt + (size_t)tix(I, J) * TB * TB + r * TB + q * 4);
        }
        for (int e = threadIdx.x; e < TB * CPR; e += blockDim.x) {
            const int r = e / CPR, q = e % CPR;
            cp_async16(Dv + r * RPB + q * 4, dinv + (size_t)J * TB * TB + r * TB + q * 4);
        }
        cp_async_wait_all();
        __syncthreads();
        float acc[4][4];
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[nt][e] = 0.f;
        if (kr > 0) mma3_rows(acc, Qw, QP, Rc, RPB, 0, kr);
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int r = g + (e >> 1) * 8, c = nt * 8 + 2 * t + (e & 1);
                const long long gr = row0 + r;
                const int gc = kr + c;
                const float y = (gr < m && gc < n) ? Y[gr + (long long)gc * ldy] : 0.f;
                Qw[r * QP + kr + c] = y - acc[nt][e];
            }
        __syncwarp();
        float o[4][4];
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int e = 0; e < 4; e++) o[nt][e] = 0.f;
        mma3_rows(o, Qw + kr, QP, Dv, RPB, 0, TB);
        __syncwarp();
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int r = g + (e >> 1) * 8, c = nt * 8 + 2 * t + (e & 1);
                Qw[r * QP + kr + c] = o[nt][e];
                const long long gr = row0 + r;
                const int gc = kr + c;
                if (gr < m && gc < n) Q[gr + (long long)gc * ldq] = o[nt][e];
            }
        __syncwarp();
    }
}

template <typename T>
constexpr int trsm_bm() { return 128; }

template <typename T>
size_t trsm_smem(int nb) {
    using S = T;
    return sizeof(S) * ((size_t)nb * TB * (trsm_bm<T>() + 4) + (size_t)nb * TB * TP + (size_t)TE);
}

}  // namespace

// G (n x n, FP64, symmetric positive definite; upper triangle read) -> R (upper, zero
// below).  When dinv is given (nb = ceil(n/32) tiles of 32 x 32, compute type), it
// receives the inverses of the diagonal tiles of R.  Returns false on breakdown
// (a pivot d_j <= rel_tol * G_jj, or not finite); d_flag is left set then.
template <typename S>
bool chol_factor(cudaStream_t s, DM<double> G, double rel_tol, int *d_flag, S *dinv) {
    const int n = (int)G.r;
    if (G.r != G.c) fail(RSVD_ERR_ARGUMENT, "cholesky: not square");
    if (n == 0) return true;
    const int nb = (n + TB - 1) / TB;
    if (!ctx().chol_deferred) RSVD_CK(cudaMemsetAsync(d_flag, 0, sizeof(int), s));
    DBuf own(dinv ? 16 : sizeof(S) * (size_t)nb * TB * TB, s);
    S *di = dinv ? dinv : (S *)own.get();
    if (nb <= smem_nb_max<S>()) {
        const size_t smem = sizeof(S) * ((size_t)(tix(0, nb) + 1) * TE + (size_t)nb * TB);
        auto k = chol_smem_kernel<S>;
        RSVD_CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<1, chol_smem_threads<S>(), smem, s>>>(G.p, G.ld, n, nb, rel_tol, di, d_flag);
        RSVD_LAUNCH_CK();
        ctx().launches++;
    } else {
        const size_t ntile = (size_t)tix(0, nb);
        DBuf wt(sizeof(S) * ntile * TB * TB, s), d0(sizeof(S) * (size_t)nb * TB, s), rd(sizeof(S) * (size_t)nb * TB * TB, s);
        S *Wt = (S *)wt.get(), *diag0 = (S *)d0.get(), *Rd = (S *)rd.get();
        const long long tot = (long long)ntile * TB * TB;
        const unsigned g = (unsigned)std::min<long long>((tot + 255) / 256, (long long)std::max(1, ctx().sms) * 16);
        chol_gload_kernel<S><<<g, 256, 0, s>>>(G.p, G.ld, n, nb, Wt, diag0);
        for (int J = 0; J < nb; J++) {
            chol_gpanel_kernel<S><<<nb - J, 32, 0, s>>>(Wt, nb, J, diag0, rel_tol, di, Rd, d_flag);
            const int nt = nb - J - 1;
            if (nt > 0) chol_gupdate_kernel<S><<<nt * (nt + 1) / 2, 32, 0, s>>>(Wt, nb, J);
        }
        const unsigned g2 = (unsigned)std::min<long long>(((long long)n * n + 255) / 256, (long long)std::max(1, ctx().sms) * 16);
        chol_gstore_kernel<S><<<g2, 256, 0, s>>>(Wt, Rd, n, G.p, G.ld);
        RSVD_LAUNCH_CK();
        ctx().launches += 2 * nb + 2;
    }
    // deferred mode: the flag stays set for the caller's one check at the end of the solve
    if (ctx().chol_deferred) return true;
    int h = 0;
    RSVD_CK(cudaMemcpyAsync(&h, d_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    RSVD_CK(cudaStreamSynchronize(s));
    return h == 0;
}

// X = R^-1 (upper, zero below), given the inverted diagonal tiles from chol_factor.
template <typename S, typename To>
void tri_inv_tiles(cudaStream_t s, DM<double> R, const S *dinv, DM<To> X) {
    const int n = (int)R.r;
    if (n == 0) return;
    const int nb = (n + TB - 1) / TB;
    const int threads = sizeof(S) == 4 ? 512 : 256, nw = threads / 32;
    const size_t smem = sizeof(S) * (size_t)(2 + 2 * nw) * TE;
    auto k = tri_inv_tiles_kernel<S, To>;
    RSVD_CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<nb, threads, smem, s>>>(R.p, R.ld, n, nb, dinv, X.p, X.ld);
    RSVD_LAUNCH_CK();
    ctx().launches++;
}

// Q = Y R^-1 by the slab solve when the slab and R's block column fit in shared memory
// (order <= 288); returns false (nothing queued) otherwise.
template <typename T>
bool trsm_right_tiles(cudaStream_t s, DM<T> Y, DM<double> R, const T *dinv, DM<T> Q) {
    const int n = (int)R.r;
    if (n == 0 || Y.r == 0) return true;
    const int nb = (n + TB - 1) / TB;
    if (nb > 9) return false;
    const size_t smem = trsm_smem<T>(nb);
    if (smem > 220 * 1024) return false;
    constexpr int BM = trsm_bm<T>();
    auto k = trsm_slab_kernel<T, T, BM>;
    RSVD_CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const long long slabs = (Y.r + BM - 1) / BM;
    if (slabs > 0x7fffffffll) fail(RSVD_ERR_ARGUMENT, "trsm: too many rows");
    k<<<(unsigned)slabs, TRSM_THREADS, smem, s>>>(Y.p, Y.ld, R.p, R.ld, nullptr, dinv, Q.p, Q.ld, Y.r, n, nb);
    RSVD_LAUNCH_CK();
    ctx().launches++;
    return true;
}

// FP32 packed-tile Cholesky (order <= 288): Gt in, R tiles out (see chol_tiles_f32_kernel).
bool chol_tiles_f32(cudaStream_t s, float *Gt, int n, double rel_tol, int *d_flag, float *dinv, DM<double> *Rout) {
    if (n == 0) return true;
    const int nb = (n + TB - 1) / TB;
    if (nb > smem_nb_max<float>()) fail(RSVD_ERR_ARGUMENT, "chol_tiles_f32: order above 288");
    if (!ctx().chol_deferred) RSVD_CK(cudaMemsetAsync(d_flag, 0, sizeof(int), s));
    const size_t smem = sizeof(float) * ((size_t)(tix(0, nb) + 1) * TE + (size_t)nb * TB);
    RSVD_CK(cudaFuncSetAttribute(chol_tiles_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    chol_tiles_f32_kernel<<<1, CHOL_F32_THREADS, smem, s>>>(Gt, n, nb, rel_tol, dinv, d_flag);
    RSVD_LAUNCH_CK();
    ctx().launches++;
    if (Rout) {
        const long long nn = (long long)n * n;
        tiles_to_fp64_kernel<<<(unsigned)std::min<long long>((nn + 255) / 256, (long long)std::max(1, ctx().sms) * 4),
                               256, 0, s>>>(Gt, n, Rout->p, Rout->ld);
        RSVD_LAUNCH_CK();
        ctx().launches++;
    }
    // deferred mode: the flag stays set for the caller's one check at the end of the solve
    if (ctx().chol_deferred) return true;
    int h = 0;
    RSVD_CK(cudaMemcpyAsync(&h, d_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    RSVD_CK(cudaStreamSynchronize(s));
    return h == 0;
}

// Q = Y R^-1 from R's packed FP32 tiles (order <= 288).
void trsm_right_tiles_f32(cudaStream_t s, DM<float> Y, int n, const float *Rt, const float *dinv, DM<float> Q) {
    if (n == 0 || Y.r == 0) return;
    const int nb = (n + TB - 1) / TB;
    if (nb > 9) fail(RSVD_ERR_ARGUMENT, "trsm_right_tiles_f32: order above 288");
    // tensor cores (3xTF32 mma.sync, one warp per 16 rows)
    const size_t smem = sizeof(float) * ((size_t)TRSM_MMA_BM * (nb * TB + 4) + (size_t)(std::max(nb - 1, 1)) * TB * RPB +
                                         (size_t)TB * RPB);
    RSVD_CK(cudaFuncSetAttribute(trsm_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const long long slabs = (Y.r + TRSM_MMA_BM - 1) / TRSM_MMA_BM;
    trsm_mma_kernel<<<(unsigned)slabs, 256, smem, s>>>(Y.p, Y.ld, Rt, dinv, Q.p, Q.ld, Y.r, n, nb);
    RSVD_LAUNCH_CK();
    ctx().launches++;
}

// Cholesky of the packed FP32 Gram and Q = Y R^-1 in one cooperative launch
// (chol_trsm_fused_kernel).  Returns -1 when the launch is not possible here (order above 288,
// or more slabs than can be co-resident: the caller runs chol_tiles_f32 and
// trsm_right_tiles_f32), else 1, or 0 on a Cholesky breakdown (undeferred mode only: deferred,
// the flag stays set for the caller's one check).  Rout (optional): R as FP64.
int chol_trsm_fused_f32(cudaStream_t s, float *Gt, int n, double rel_tol, float *dinv, DM<double> *Rout, DM<float> Y,
                        DM<float> Q) {
    if (n == 0 || Y.r == 0) return -1;
    const int nb = (n + TB - 1) / TB;
    if (nb > smem_nb_max<float>()) return -1;
    const long long slabs = (Y.r + TRSM_MMA_BM - 1) / TRSM_MMA_BM;
    const size_t smem_chol = sizeof(float) * ((size_t)(tix(0, nb) + 1) * TE + (size_t)nb * TB);
    const size_t smem_trsm = sizeof(float) * ((size_t)TRSM_MMA_BM * (nb * TB + 4) +
                                              (size_t)std::max(nb - 1, 1) * TB * RPB + (size_t)TB * RPB);
    const size_t smem = std::max(smem_chol, smem_trsm);
    int dev = 0, coop = 0;
    RSVD_CK(cudaGetDevice(&dev));
    RSVD_CK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return -1;
    RSVD_CK(cudaFuncSetAttribute(chol_trsm_fused_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    RSVD_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chol_trsm_fused_kernel, 256, smem));
    if ((long long)per_sm * std::max(1, ctx().sms) < slabs + 1) return -1;
    int *flags = ctx().d_flags;
    if (!ctx().chol_deferred) RSVD_CK(cudaMemsetAsync(flags + FLAG_CHOL_BREAKDOWN, 0, sizeof(int), s));
    DBuf rb(sizeof(int) * (size_t)nb, s);
    int *ready = (int *)rb.get();
    RSVD_CK(cudaMemsetAsync(ready, 0, sizeof(int) * (size_t)nb, s));
    const float *yp = Y.p;
    long long ldy = Y.ld, ldq = Q.ld, m = Y.r;
    float *qp = Q.p;
    void *args[] = {(void *)&Gt, (void *)&n, (void *)&nb, (void *)&rel_tol, (void *)&dinv, (void *)&flags,
                    (void *)&ready, (void *)&yp, (void *)&ldy, (void *)&qp, (void *)&ldq, (void *)&m};
    RSVD_CK(cudaLaunchCooperativeKernel((const void *)chol_trsm_fused_kernel, dim3((unsigned)(slabs + 1)), dim3(256),
                                        args, smem, s));
    RSVD_LAUNCH_CK();
    ctx().launches++;
    if (Rout) {
        const long long nn = (long long)n * n;
        tiles_to_fp64_kernel<<<(unsigned)std::min<long long>((nn + 255) / 256, (long long)std::max(1, ctx().sms) * 4),
                               256, 0, s>>>(Gt, n, Rout->p, Rout->ld);
        RSVD_LAUNCH_CK();
        ctx().launches++;
    }
    if (ctx().chol_deferred) return 1;
    int h = 0;
    RSVD_CK(cudaMemcpyAsync(&h, flags + FLAG_CHOL_BREAKDOWN, sizeof(int), cudaMemcpyDeviceToHost, s));
    RSVD_CK(cudaStreamSynchronize(s));
    return h == 0 ? 1 : 0;
}

// C = A B (FP32, column-major) by 3xTF32 on the tensor cores (gemm_nn_3xtf32_kernel).
void gemm_nn_3xtf32(cudaStream_t s, DM<float> A, DM<float> B, DM<float> C) {
    const int M = (int)A.r, K = (int)A.c, N = (int)B.c;
    if (B.r != K || C.r != M || C.c != N) fail(RSVD_ERR_ARGUMENT, "gemm_nn_3xtf32: shapes");
    if (M == 0 || N == 0) return;
    const size_t smem = sizeof(uint32_t) * 2 * ((size_t)G3_BM * G3_AP + (size_t)G3_BK * G3_BP);
    RSVD_CK(cudaFuncSetAttribute(gemm_nn_3xtf32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const dim3 grid((unsigned)((M + G3_BM - 1) / G3_BM), (unsigned)((N + G3_BN - 1) / G3_BN));
    gemm_nn_3xtf32_kernel<<<grid, 256, smem, s>>>(A.p, A.ld, B.p, B.ld, C.p, C.ld, M, N, K);
    RSVD_LAUNCH_CK();
    ctx().launches++;
}

template <typename S>
void tri_mul_upper(cudaStream_t s, DM<double> A, DM<double> B, DM<double> C) {
    const int n = (int)A.r;
    if (n == 0) return;
    const int nb = (n + TB - 1) / TB;
    const int tiles = nb * nb;     // upper tiles + strictly lower tiles (zeroed)
    tri_mul_upper_kernel<S><<<tiles, 256, 0, s>>>(A.p, A.ld, B.p, B.ld, C.p, C.ld, n, nb);
    RSVD_LAUNCH_CK();
    ctx().launches++;
}

template bool chol_factor<float>(cudaStream_t, DM<double>, double, int *, float *);
template bool chol_factor<double>(cudaStream_t, DM<double>, double, int *, double *);
template void tri_inv_tiles<float, float>(cudaStream_t, DM<double>, const float *, DM<float>);
template void tri_inv_tiles<float, double>(cudaStream_t, DM<double>, const float *, DM<double>);
template void tri_inv_tiles<double, double>(cudaStream_t, DM<double>, const double *, DM<double>);
template bool trsm_right_tiles<float>(cudaStream_t, DM<float>, DM<double>, const float *, DM<float>);
template bool trsm_right_tiles<double>(cudaStream_t, DM<double>, DM<double>, const double *, DM<double>);
template void tri_mul_upper<float>(cudaStream_t, DM<double>, DM<double>, DM<double>);
template void tri_mul_upper<double>(cudaStream_t, DM<double>, DM<double>, DM<double>);

}  // namespace rsvd
