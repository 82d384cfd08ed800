// k_small.cu -- the k x k (l x l) steps of every decomposition, templated on the compute
// type S: S = double in the FP64 mode (reproduces the reference), S = float in the mixed
// modes.  Storage is FP64 throughout; S only sets the arithmetic.
//
// Why two compute types: GB300 executes FP64 at ~2 FMA/clock/SM (cuBLAS DGEMM measures
// 1.1 TFLOP/s on the whole GPU), so an l x l factorisation that runs on one SM costs
// milliseconds in FP64 and tens of microseconds in FP32.  In the mixed modes the inputs
// of these steps (Grams of FP32 data) are only FP32-accurate anyway.
//
//   cholesky_small  : G = R^T R through the tiled factorisation of k_chol.cu
//   jacobi_small    : one-sided Jacobi SVD, one CTA, round-robin pair ordering
#include "rsvd_internal.h"
#include "k_common.cuh"

#include <algorithm>
#include <climits>
#include <cmath>
#include <limits>
#include <type_traits>

#include <cooperative_groups.h>

namespace rsvd {

namespace {

template <typename S>
__device__ __forceinline__ S warp_sum_t(S v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
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

// Jacobi rotation (cs, sn) zeroing w_p.w_q = d, |w_p|^2 = a, |w_q|^2 = b (Rutishauser's
// formulas); FP32 with correctly rounded reciprocal / rsqrt intrinsics instead of the
// division and square-root sequences.
// FP32: the tangent t only has to annihilate the pair to about FP32 precision, so it takes the
// hardware's approximate reciprocal and reciprocal square root (the correctly rounded sequences
// sat on the round's critical path); the cosine, whose rounding decides how orthogonal the
// accumulated rotations stay, is correctly rounded (an approximate cosine with one Newton step
// drifted the column norms by ~1e-4 over a 272-column solve).
__device__ __forceinline__ void jrot_t(float a, float b, float d, float &cs, float &sn, float &t) {
    const float zeta = __fdividef(b - a, 2.f * d);
    const float az = fabsf(zeta);
    if (az < 1e18f) {
        const float z2 = fmaf(zeta, zeta, 1.f);
        t = copysignf(__fdividef(1.f, fmaf(z2, rsqrtf(z2), az)), zeta);      // 1 / (|z| + sqrt(1 + z^2))
    } else {
        t = __fdividef(0.5f, zeta);
    }
    cs = __frsqrt_rn(fmaf(t, t, 1.f));
    sn = cs * t;
}
__device__ __forceinline__ void jrot(float a, float b, float d, float &cs, float &sn) {
    float t;
    jrot_t(a, b, d, cs, sn, t);
}
__device__ __forceinline__ void jrot(double a, double b, double d, double &cs, double &sn) {
    const double zeta = (b - a) / (2.0 * d);
    const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
    cs = 1.0 / sqrt(1.0 + t * t);
    sn = cs * t;
}
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Block-cyclic one-sided Jacobi on a cluster of CLN CTAs (8, or 16 where the GPU can
// co-schedule a non-portable cluster of 16).  The n columns of W and V are cut into
// NBLK = 2 CLN blocks of bs columns.  CTA i holds the blocks at tournament positions i
// (slot 0) and NBLK-1-i (slot 1), whole columns (all n rows) of W and V, in shared memory.
// A super-round orthogonalises every pair among the CTA's 2*bs columns (one cyclic inner
// sweep, block barriers only); then positions 1..NBLK-1 rotate by one (position 0 stays)
// and every block moves to its next holder as one bulk asynchronous copy into the holder's
// shared memory (completing on the holder's mbarrier, waited with a bound), followed by one
// cluster barrier.  NBLK-1 super-rounds meet every pair of blocks once: one outer sweep.
// Outer sweeps repeat until no CTA rotated anything during a whole sweep, or (FP32) until
// the largest cos^2 = (w_p.w_q)^2 / (|w_p|^2 |w_q|^2) seen in a sweep is below stop_tol.  The
// caller passes tol / 10: quadratic convergence would make cos^2 < tol enough for the next
// sweep to find every pair below tol, but clustered singular values converge more slowly, and
// on 272-column factors of the 16384 x 8192 workload that shortcut stopped one sweep early on
// some sketches, leaving hundreds of nearly-equal pairs to the refinement's sequential rotations.
// Each warp keeps its rotation count and largest cos^2 in registers during a sweep (no
// shared-memory atomics in the rounds) and folds them into the CTA's totals at its end.
// One warp per pair (blockDim = 32 bs, at most 16 warps so that the register-held chunks
// fit): a lane keeps its 16-byte chunks of w_p and w_q in registers between the dot
// products and the rotation (MAXIT chunks: ldr <= 32 MAXIT VW); FP32 uses packed FFMA2.
// Shared memory per CTA: 2 buffers x 2 slots x bs x ldr x 2 (W, V) x sizeof(S).
template <typename S, int CLN>
__global__ void __launch_bounds__(512, 1) jacobi_block_cluster_kernel(const double *G, long long ldg, int n, int bs,
                                                                    int ldr, S tol, S stop_tol, int max_sweeps, S *Wout,
                                                                    S *Vout, long long ldo, int *sweeps_out, int *flag) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    constexpr int NBLK = 2 * CLN;
    constexpr int VW = 16 / sizeof(S);
    constexpr int MAXIT = sizeof(S) == 4 ? 4 : 8;
    using V16 = typename std::conditional<sizeof(S) == 4, float4, double2>::type;
    extern __shared__ __align__(16) unsigned char shraw[];
    const size_t slot_elems = (size_t)bs * ldr * 2;          // W columns then V columns
    S *buf = (S *)shraw;                                      // [2 buffers][2 slots][slot_elems]
    __shared__ int blk[2][2];                                 // block id held in [buffer][slot]
    __shared__ int rot_count;
    __shared__ int sweep_rot[CLN];
    __shared__ unsigned char ftab[64][32][2];                 // full-round pairs (p < q), nloc <= 64
    __shared__ __align__(8) unsigned long long inbar;         // incoming block copies
    __shared__ unsigned int sweep_max;                        // largest cos^2 of the sweep (float bits)
    __shared__ unsigned int cl_max[CLN];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    auto slot_ptr = [&](S *base, int b, int sl) { return base + ((size_t)b * 2 + sl) * slot_elems; };
    auto col_w = [&](S *sp, int j) { return sp + (size_t)j * ldr; };
    auto col_v = [&](S *sp, int j) { return sp + (size_t)(bs + j) * ldr; };
    const int nloc = 2 * bs;                 // local columns (even)

    // initial placement: slot 0 <- block rank, slot 1 <- block NBLK-1-rank; pair table
    if (threadIdx.x == 0) {
        blk[0][0] = rank;
        blk[0][1] = NBLK - 1 - rank;
        rot_count = 0;
        sweep_max = 0u;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&inbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int e = threadIdx.x; e < (nloc - 1) * bs; e += blockDim.x) {
        const int r = e / bs, pi = e % bs;
        int p, q;
        rr_pair2(nloc, r, pi, p, q);
        if (p > q) { const int t = p; p = q; q = t; }
        ftab[r][pi][0] = (unsigned char)p;
        ftab[r][pi][1] = (unsigned char)q;
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
    uint32_t mphase = 0;
    const int nvec = ldr / VW;               // columns are zero beyond n up to ldr (a multiple of 4)
    const uint32_t slot_bytes = (uint32_t)(slot_elems * sizeof(S));
    float wmax = 0.f;                        // this warp's largest cos^2 and rotations in the sweep
    int wrot = 0;
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
                for (int pi = wid; pi < bs; pi += nw) {
                    int p, q;
                    if (full) {
                        p = ftab[r][pi][0];
                        q = ftab[r][pi][1];
                    } else {
                        p = pi;
                        const int t = pi + r;
                        q = bs + (t >= bs ? t - bs : t);
                    }
                    // skip padding columns beyond n
                    const int gp = (p < bs) ? b0 * bs + p : b1 * bs + (p - bs);
                    const int gq = (q < bs) ? b0 * bs + q : b1 * bs + (q - bs);
                    if (gp >= n || gq >= n) continue;
                    V16 *wp = reinterpret_cast<V16 *>((p < bs) ? col_w(s0, p) : col_w(s1, p - bs));
                    V16 *wq = reinterpret_cast<V16 *>((q < bs) ? col_w(s0, q) : col_w(s1, q - bs));
                    V16 xr[MAXIT], yr[MAXIT];
                    S a = 0, b = 0, d = 0;
                    if constexpr (sizeof(S) == 4) {
                        // packed FP32 pairs (FFMA2): half the FMA instructions
                        float2 a2 = make_float2(0.f, 0.f), b2 = a2, d2 = a2;
#pragma unroll
                        for (int it = 0; it < MAXIT; it++) {
                            const int iv = lane + 32 * it;
                            if (iv < nvec) {
                                xr[it] = wp[iv];
                                yr[it] = wq[iv];
                                const float2 x0 = make_float2(xr[it].x, xr[it].y), x1 = make_float2(xr[it].z, xr[it].w);
                                const float2 y0 = make_float2(yr[it].x, yr[it].y), y1 = make_float2(yr[it].z, yr[it].w);
                                a2 = __ffma2_rn(x0, x0, a2); a2 = __ffma2_rn(x1, x1, a2);
                                b2 = __ffma2_rn(y0, y0, b2); b2 = __ffma2_rn(y1, y1, b2);
                                d2 = __ffma2_rn(x0, y0, d2); d2 = __ffma2_rn(x1, y1, d2);
                            }
                        }
                        a = a2.x + a2.y; b = b2.x + b2.y; d = d2.x + d2.y;
                    } else {
#pragma unroll
                        for (int it = 0; it < MAXIT; it++) {
                            const int iv = lane + 32 * it;
                            if (iv < nvec) {
                                xr[it] = wp[iv];
                                yr[it] = wq[iv];
                                const S *x = reinterpret_cast<const S *>(&xr[it]), *y = reinterpret_cast<const S *>(&yr[it]);
#pragma unroll
                                for (int e = 0; e < VW; e++) {
                                    a = fma(x[e], x[e], a); b = fma(y[e], y[e], b); d = fma(x[e], y[e], d);
                                }
                            }
                        }
                    }
                    a = warp_sum_t(a); b = warp_sum_t(b); d = warp_sum_t(d);
                    const S ab = a * b, dd = d * d;
                    if (ab > S(0)) wmax = fmaxf(wmax, __fdividef((float)dd, (float)ab));
                    if (d == S(0) || dd <= tol * tol * ab) continue;
                    S cs, sn;
                    jrot(a, b, d, cs, sn);
                    V16 *vp = reinterpret_cast<V16 *>((p < bs) ? col_v(s0, p) : col_v(s1, p - bs));
                    V16 *vq = reinterpret_cast<V16 *>((q < bs) ? col_v(s0, q) : col_v(s1, q - bs));
#pragma unroll
                    for (int it = 0; it < MAXIT; it++) {
                        const int iv = lane + 32 * it;
                        if (iv < nvec) {
                            V16 uv = vp[iv], vv = vq[iv];
                            if constexpr (sizeof(S) == 4) {
                                // (x, y) <- (cs x - sn y, sn x + cs y) on packed pairs
                                const float2 c2 = make_float2(cs, cs), s2 = make_float2(sn, sn);
                                const float2 ns2 = make_float2(-sn, -sn);
                                auto rot = [&](float &p0, float &p1, float &q0, float &q1) {
                                    const float2 pp = make_float2(p0, p1), qq = make_float2(q0, q1);
                                    const float2 np = __ffma2_rn(c2, pp, __fmul2_rn(ns2, qq));
                                    const float2 nq = __ffma2_rn(s2, pp, __fmul2_rn(c2, qq));
                                    p0 = np.x; p1 = np.y; q0 = nq.x; q1 = nq.y;
                                };
                                rot(xr[it].x, xr[it].y, yr[it].x, yr[it].y);
                                rot(xr[it].z, xr[it].w, yr[it].z, yr[it].w);
                                rot(uv.x, uv.y, vv.x, vv.y);
                                rot(uv.z, uv.w, vv.z, vv.w);
                            } else {
                                S *x = reinterpret_cast<S *>(&xr[it]), *y = reinterpret_cast<S *>(&yr[it]);
                                S *u = reinterpret_cast<S *>(&uv), *v = reinterpret_cast<S *>(&vv);
#pragma unroll
                                for (int e = 0; e < VW; e++) {
                                    const S x0 = x[e], y0 = y[e], u0 = u[e], v0 = v[e];
                                    x[e] = cs * x0 - sn * y0;
                                    y[e] = sn * x0 + cs * y0;
                                    u[e] = cs * u0 - sn * v0;
                                    v[e] = sn * u0 + cs * v0;
                                }
                            }
                            wp[iv] = xr[it];
                            wq[iv] = yr[it];
                            vp[iv] = uv;
                            vq[iv] = vv;
                        }
                    }
                    wrot++;
                }
                __syncthreads();
            }
            // ---- move blocks to their next holders (positions 1..NBLK-1 rotate by one)
            const int nxt = cur ^ 1;
            int dst0, dsl0, dst1, dsl1;       // destination (cta, slot) of local slots 0 and 1
            if (rank == 0) { dst0 = 0; dsl0 = 0; }
            else if (rank < CLN - 1) { dst0 = rank + 1; dsl0 = 0; }
            else { dst0 = CLN - 1; dsl0 = 1; }
            if (rank == 0) { dst1 = 1; dsl1 = 0; }
            else { dst1 = rank - 1; dsl1 = 1; }
            // the rounds' generic-proxy writes of the outgoing slots, then the copies
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            if (threadIdx.x == 0) {
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(&inbar)),
                             "r"(2u * slot_bytes)
                             : "memory");
                for (int sl = 0; sl < 2; sl++) {
                    const int dc = sl ? dst1 : dst0, ds = sl ? dsl1 : dsl0;
                    uint32_t rdst, rbar;
                    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(rdst) : "r"(smem_addr(slot_ptr(buf, nxt, ds))), "r"(dc));
                    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(rbar) : "r"(smem_addr(&inbar)), "r"(dc));
                    asm volatile(
                        "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(rdst),
                        "r"(smem_addr(slot_ptr(buf, cur, sl))), "r"(slot_bytes), "r"(rbar)
                        : "memory");
                    int *rb = cluster.map_shared_rank(&blk[nxt][ds], dc);
                    *rb = sl ? b1 : b0;
                }
            }
            // both incoming slots (bounded wait: ~1 s of SM cycles, then the error flag)
            {
                uint32_t ok = 0;
                const long long t0 = clock64();
                while (true) {
                    asm volatile(
                        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                        "selp.u32 %0, 1, 0, p;\n\t}\n"
                        : "=r"(ok)
                        : "r"(smem_addr(&inbar)), "r"(mphase)
                        : "memory");
                    if (ok) break;
                    if (clock64() - t0 > (1ll << 31)) { atomicExch(flag, 1); break; }
                }
                mphase ^= 1u;
            }
            cluster.sync();
            cur = nxt;
        }
        // ---- did any CTA rotate during this sweep, and how large was the largest cosine?
        if (lane == 0) {
            atomicMax(&sweep_max, __float_as_uint(wmax));
            atomicAdd(&rot_count, wrot);
        }
        wmax = 0.f;
        wrot = 0;
        __syncthreads();
        if (threadIdx.x < CLN) {
            int *dstf = cluster.map_shared_rank(&sweep_rot[rank], (unsigned)threadIdx.x);
            *dstf = rot_count;
            unsigned int *dstm = cluster.map_shared_rank(&cl_max[rank], (unsigned)threadIdx.x);
            *dstm = sweep_max;
        }
        cluster.sync();
        int total = 0;
        float cmax = 0.f;
#pragma unroll
        for (int c = 0; c < CLN; c++) {
            total += sweep_rot[c];
            cmax = fmaxf(cmax, __uint_as_float(cl_max[c]));
        }
        __syncthreads();
        if (threadIdx.x == 0) { rot_count = 0; sweep_max = 0u; }
        cluster.sync();
        if (total == 0) break;
        // FP32 only: |cos| < sqrt(tol) (cos^2 < tol).  FP64 keeps the plain criterion, so that
        // its factors match the reference's to the last sweep.
        if (sizeof(S) == 4 && (double)cmax < (double)stop_tol) { sweep++; break; }
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

// FP32 block-cyclic Jacobi, register-resident Gram form, for a fixed block width BS (the
// cluster layout, pair schedule and convergence tests of jacobi_block_cluster_kernel; its block
// moves with a split cluster barrier, see the kernel).  A super-round of the one-sided kernel
// costs one block barrier, two n-row passes and three warp reductions per round; here it is
// three phases:
//   Gram   Gl = P^T P of the CTA's NL = 2 BS local columns P (n rows), all warps: TK x TK
//          output blocks x row slices (consecutive lanes take consecutive 16-byte row chunks),
//          partial sums reduced through shared memory;
//   rounds lane i of warp 0 holds row i of Gl, lane i of warp 1 row i of Z (the accumulated
//          rotation), in registers, with fixed pair positions and the columns moved between
//          rounds so that every register index is static (gr_rounds_g / gr_rounds_z).  A round:
//          lane l < BS of warp 0 computes the rotation of pair l from Gl_pp, Gl_qq, Gl_pq, the
//          rotations are broadcast (shuffles within warp 0, shared memory and a named barrier
//          to warp 1), the column rotations are applied to the rows of Gl and Z and the row
//          rotation of Gl by exchanging rows with the partner lane; the diagonal block takes
//          a' = a - t d, b' = b + t d, d' = 0.
//   apply  P <- P Z for the W and V columns: one thread per 4-row chunk of one matrix, Z rows
//          broadcast from shared memory, 4 x NL accumulators (skipped when nothing rotated).
// Gl is formed afresh at every super-round, so the rounding of the two-sided updates does not
// accumulate; its FP32 dot products carry the one-sided kernel's ~sqrt(n) eps relative error.
// The super-round's rounds on two warps in lockstep.  Warp 0: lane i < 2 BS holds row i of Gl
// (g) for the columns at positions 0..2 BS-1 and dg = Gl_ii; warp 1: lane i holds row i of Z.
// The pairs sit at fixed positions -- cross rounds (k, BS + k), the full round of a sweep's first
// super-round (k, 2 BS - 1 - k) -- and the columns move between rounds instead: cross rounds
// shift positions BS..2 BS-1 down by one, full rounds rotate positions 1..2 BS-1 (the circle
// method).  So every register index is static inside one compact loop body (a loop unrolled over
// the rounds did not fit the instruction cache).  Column moves are register moves within a lane,
// row moves (Gl only) are shuffles between lanes; after the last round every column is back at
// its starting position.  A round: lane k < BS of warp 0 computes the rotation of pair k from dg
// and Gl(k, partner) and publishes it (cos, sin, ballot) in shared memory, double-buffered by
// round parity; a named barrier over the two warps hands it to warp 1, which rotates the columns
// of Z while warp 0 rotates its rows of Gl by columns, then takes its next row in one exchange:
// the row rotation against the partner's row and the row and column moves fused (two shuffles
// an entry, from the lane whose row moves here and from that lane's partner).  Only the
// rotated pair's diagonal is updated exactly (a' = a - t d, b' = b + t d); its off-diagonal entry
// keeps the rounding of the general formula, which is never read again in the super-round (each
// pair meets once) and is recomputed at the next one.  Adjacent pairs are rotated as packed
// FP32 pairs (FFMA2).
// Position k's next occupant: a full round rotates positions 1..2 BS-1 by one (the circle
// method), a cross round positions BS..2 BS-1; used for columns (registers) and rows (lanes).
template <int BS, bool FULLR>
__host__ __device__ constexpr int gr_next(int k) {
    return FULLR ? (k == 0 ? 0 : (k == 2 * BS - 1 ? 1 : k + 1)) : (k < BS ? k : (k == 2 * BS - 1 ? BS : k + 1));
}
template <int BS, bool FULLR>
__device__ __forceinline__ void gr_move(float (&g)[2 * BS]) {
    constexpr int NL = 2 * BS;
    if (FULLR) {
        const float g1 = g[1];
#pragma unroll
        for (int k = 1; k < NL - 1; k++) g[k] = g[k + 1];
        g[NL - 1] = g1;
    } else {
        const float g0 = g[BS];
#pragma unroll
        for (int k = BS; k < NL - 1; k++) g[k] = g[k + 1];
        g[NL - 1] = g0;
    }
}
// column rotations of one row: new col p = c col_p - s col_q, new col q = s col_p + c col_q,
// pairs k and k + 1 packed
template <int BS, bool FULLR>
__device__ __forceinline__ void gr_colrot(float (&g)[2 * BS], const float *C, const float *Sn) {
    constexpr int NL = 2 * BS;
#pragma unroll
    for (int k = 0; k + 1 < BS; k += 2) {
        const int P0 = k, Q0 = FULLR ? NL - 1 - k : BS + k;
        const int P1 = k + 1, Q1 = FULLR ? NL - 2 - k : BS + k + 1;
        const float2 c2 = make_float2(C[k], C[k + 1]), s2 = make_float2(Sn[k], Sn[k + 1]);
        const float2 xp = make_float2(g[P0], g[P1]), xq = make_float2(g[Q0], g[Q1]);
        const float2 np = __ffma2_rn(c2, xp, __fmul2_rn(make_float2(-s2.x, -s2.y), xq));
        const float2 nq = __ffma2_rn(s2, xp, __fmul2_rn(c2, xq));
        g[P0] = np.x; g[P1] = np.y; g[Q0] = nq.x; g[Q1] = nq.y;
    }
    if (BS % 2) {
        constexpr int k = BS - 1;
        const int P = k, Q = FULLR ? NL - 1 - k : BS + k;
        const float xp = g[P], xq = g[Q];
        g[P] = fmaf(C[k], xp, -Sn[k] * xq);
        g[Q] = fmaf(Sn[k], xp, C[k] * xq);
    }
}
template <int BS, bool FULLR>
__device__ __forceinline__ void gr_rounds_g(float (&g)[2 * BS], float &dg, int lane, int b0, int b1, int n, float tol,
                                            float &wmax, int &wrot, bool &any, float *rot_cs, float *rot_sn,
                                            unsigned int *rot_bal) {
    constexpr int NL = 2 * BS;
    constexpr int NR = FULLR ? NL - 1 : BS;
    const int partner = lane >= NL ? lane : (FULLR ? NL - 1 - lane : (lane < BS ? lane + BS : lane - BS));
    const int src = lane >= NL ? lane
                    : (FULLR ? (lane == 0 ? 0 : (lane % (NL - 1)) + 1)
                             : (lane < BS ? lane : BS + (lane - BS + 1) % BS));
    // the row this lane takes next is the rotated row of lane src: c_src row_src +- s_src row_psrc
    const int psrc = src >= NL ? src : (FULLR ? NL - 1 - src : (src < BS ? src + BS : src - BS));
    const int pidx_s = src >= NL ? 0 : (FULLR ? (src < BS ? src : NL - 1 - src) : (src < BS ? src : src - BS));
    const bool isp_s = src < BS;
#pragma unroll 1
    for (int r = 0; r < NR; r++) {
        float op = 0.f;                                   // Gl(lane, partner)
#pragma unroll
        for (int k = 0; k < BS; k++) {
            const int P = k, Q = FULLR ? NL - 1 - k : BS + k;
            if (lane == P) op = g[Q];
            if (lane == Q) op = g[P];
        }
        const float b = __shfl_sync(0xffffffffu, dg, partner);
        const float a = dg, d = op;
        int op_, oq_;                                     // original columns at the pair's positions
        if (FULLR) {
            op_ = lane == 0 ? 0 : ((lane - 1 + r) % (NL - 1)) + 1;
            oq_ = ((partner - 1 + r) % (NL - 1)) + 1;
        } else {
            op_ = lane;
            oq_ = BS + (lane + r) % BS;
        }
        const int gp = (op_ < BS) ? b0 * BS + op_ : b1 * BS + (op_ - BS);
        const int gq = (oq_ < BS) ? b0 * BS + oq_ : b1 * BS + (oq_ - BS);
        float cs = 1.f, sn = 0.f, t = 0.f;
        bool act = false;
        unsigned int c2 = 0u;
        if (lane < BS && gp < n && gq < n) {
            const float ab = a * b, dd = d * d;
            if (ab > 0.f) c2 = __float_as_uint(__fdividef(dd, ab));
            if (d != 0.f && dd > tol * tol * ab) {
                jrot_t(a, b, d, cs, sn, t);
                act = true;
            }
        }
        const unsigned int bal = __ballot_sync(0xffffffffu, act);
        const int slot = r & 1;
        if (lane < BS) {
            rot_cs[slot * BS + lane] = cs;
            rot_sn[slot * BS + lane] = sn;
        }
        if (lane == 0) rot_bal[slot] = bal;
        asm volatile("bar.sync 1, 64;" ::: "memory");      // hand the round to warp 1
        wmax = fmaxf(wmax, __uint_as_float(__reduce_max_sync(0xffffffffu, c2)));
        if (bal != 0u) {
            wrot += __popc(bal);
            any = true;
            const float dgp = fmaf(-t, d, a), dgq = fmaf(t, d, b);
            float C[BS], Sn[BS];
#pragma unroll
            for (int k = 0; k < BS; k++) {
                C[k] = __shfl_sync(0xffffffffu, cs, k);
                Sn[k] = __shfl_sync(0xffffffffu, sn, k);
            }
            const float c_s = __shfl_sync(0xffffffffu, cs, pidx_s), s_s = __shfl_sync(0xffffffffu, sn, pidx_s);
            const float dp_s = __shfl_sync(0xffffffffu, dgp, pidx_s), dq_s = __shfl_sync(0xffffffffu, dgq, pidx_s);
            const float dg_s = __shfl_sync(0xffffffffu, dg, src);
            const bool act_s = src < NL && ((bal >> pidx_s) & 1u);
            gr_colrot<BS, FULLR>(g, C, Sn);
            // row rotation (J^T Gl) and the move in one exchange: position k of the next row is
            // column gr_next(k) of src's rotated row, c row_src -+ s row_psrc (the arithmetic
            // lane src would have done itself)
            const float cr = act_s ? c_s : 1.f, sr = act_s ? (isp_s ? -s_s : s_s) : 0.f;
            const float2 cr2 = make_float2(cr, cr), sr2 = make_float2(sr, sr);
            float ng[NL];
#pragma unroll
            for (int k = 0; k < NL; k += 2) {
                const int m0 = gr_next<BS, FULLR>(k), m1 = gr_next<BS, FULLR>(k + 1);
                const float x0 = __shfl_sync(0xffffffffu, g[m0], src), x1 = __shfl_sync(0xffffffffu, g[m1], src);
                const float o0 = __shfl_sync(0xffffffffu, g[m0], psrc), o1 = __shfl_sync(0xffffffffu, g[m1], psrc);
                const float2 nv = __ffma2_rn(cr2, make_float2(x0, x1), __fmul2_rn(sr2, make_float2(o0, o1)));
                ng[k] = nv.x;
                ng[k + 1] = nv.y;
            }
#pragma unroll
            for (int k = 0; k < NL; k++) g[k] = ng[k];
            dg = act_s ? (isp_s ? dp_s : dq_s) : dg_s;
        } else {
            float ng[NL];
#pragma unroll
            for (int k = 0; k < NL; k++) ng[k] = __shfl_sync(0xffffffffu, g[gr_next<BS, FULLR>(k)], src);
#pragma unroll
            for (int k = 0; k < NL; k++) g[k] = ng[k];
            dg = __shfl_sync(0xffffffffu, dg, src);
        }
    }
}
template <int BS, bool FULLR>
__device__ __forceinline__ void gr_rounds_z(float (&z)[2 * BS], const float *rot_cs, const float *rot_sn,
                                            const unsigned int *rot_bal) {
    constexpr int NL = 2 * BS;
    constexpr int NR = FULLR ? NL - 1 : BS;
#pragma unroll 1
    for (int r = 0; r < NR; r++) {
        asm volatile("bar.sync 1, 64;" ::: "memory");      // round r published by warp 0
        const int slot = r & 1;
        if (rot_bal[slot] != 0u) {
            float C[BS], Sn[BS];
#pragma unroll
            for (int k = 0; k < BS; k++) {
                C[k] = rot_cs[slot * BS + k];
                Sn[k] = rot_sn[slot * BS + k];
            }
            gr_colrot<BS, FULLR>(z, C, Sn);
        }
        gr_move<BS, FULLR>(z);
    }
}

// P <- P Z for the W and V columns of a super-round (in place): one thread per 4-row chunk of
// one matrix, 4 x 2 BS accumulators, Z rows (pitch 2 BS + 2) broadcast from shared memory.
// Not inlined, so that its accumulators and warp 0's register rounds are allocated apart.
template <int BS>
__device__ __noinline__ void gr_apply(float *s0, float *s1, int ldr, int nch, const float *zs) {
    constexpr int NL = 2 * BS, ZP = NL + 2;
    for (int task = threadIdx.x; task < 2 * nch; task += blockDim.x) {
        const bool isv = task >= nch;
        const int ch = isv ? task - nch : task;
        // column c of W: c < BS in slot 0, else slot 1; V columns follow the W columns of a slot
        auto col = [&](int c) {
            return (c < BS) ? s0 + (size_t)((isv ? BS : 0) + c) * ldr : s1 + (size_t)((isv ? BS : 0) + c - BS) * ldr;
        };
        float2 y[4][NL / 2];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int j = 0; j < NL / 2; j++) y[a][j] = make_float2(0.f, 0.f);
#pragma unroll
        for (int i = 0; i < NL; i++) {
            const float4 x = *reinterpret_cast<const float4 *>(col(i) + 4 * ch);
            const float xs[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
            for (int j = 0; j < NL / 2; j++) {
                const float2 zz = *reinterpret_cast<const float2 *>(zs + i * ZP + 2 * j);
#pragma unroll
                for (int a = 0; a < 4; a++) y[a][j] = __ffma2_rn(make_float2(xs[a], xs[a]), zz, y[a][j]);
            }
        }
#pragma unroll
        for (int j = 0; j < NL / 2; j++) {
            *reinterpret_cast<float4 *>(col(2 * j) + 4 * ch) = make_float4(y[0][j].x, y[1][j].x, y[2][j].x, y[3][j].x);
            *reinterpret_cast<float4 *>(col(2 * j + 1) + 4 * ch) = make_float4(y[0][j].y, y[1][j].y, y[2][j].y, y[3][j].y);
        }
    }
}

constexpr int GR_THREADS = 256;   // 8 warps: up to 255 registers a thread for warp 0's register rounds

// Block held in slot sl of CTA `rank` after s moves of a sweep: slot 0 is tournament position
// rank, slot 1 position nblk-1-rank; position 0 keeps block 0 and positions 1..nblk-1 rotate by
// one per move, so a sweep's nblk-1 moves bring every block back to its starting position.
__device__ __forceinline__ int gr_block(int rank, int sl, int s, int nblk) {
    const int pos = sl == 0 ? rank : nblk - 1 - rank, m = nblk - 1;
    return pos == 0 ? 0 : ((pos - 1 - s) % m + m) % m + 1;
}
// The split cluster barrier of the block moves (all threads, warp-uniform).
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }
template <int CLN, int BS>
__global__ void __launch_bounds__(GR_THREADS, 1) jacobi_gramreg_kernel(const double *G, long long ldg, int n, int ldr,
                                                               float tol, float stop_tol, int max_sweeps, float *Wout,
                                                               float *Vout, long long ldo, int *sweeps_out, int *flag) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    constexpr int NBLK = 2 * CLN;
    constexpr int NL = 2 * BS;
    constexpr int TK = (NL % 3 == 0) ? 3 : 2;                 // Gram output blocks TK x TK
    constexpr int NT = NL / TK, NTP = NT * (NT + 1) / 2;
    constexpr int KS0 = GR_THREADS / NTP, KS = (KS0 % 2 == 0) ? KS0 - 1 : KS0;   // row slices (odd: conflict-free reduction)
    constexpr int bs = BS;
    extern __shared__ __align__(16) unsigned char shraw[];
    const size_t slot_elems = (size_t)bs * ldr * 2;          // W columns then V columns
    float *buf = (float *)shraw;                              // [2 buffers][2 slots][slot_elems]
    __shared__ int rot_count, sr_rot;
    __shared__ int sweep_rot[CLN];
    __shared__ __align__(8) unsigned long long inbar;
    __shared__ unsigned int sweep_max;
    __shared__ unsigned int cl_max[CLN];
    __shared__ float gsm[NL][NL + 1];
    __shared__ __align__(16) float zsm[NL][NL + 2];
    __shared__ float red[KS * NTP * TK * TK];
    __shared__ float rot_cs[2 * BS], rot_sn[2 * BS];          // a round's rotations, by round parity
    __shared__ unsigned int rot_bal[2];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    auto slot_ptr = [&](float *base, int b, int sl) { return base + ((size_t)b * 2 + sl) * slot_elems; };

    if (threadIdx.x == 0) {
        rot_count = 0;
        sweep_max = 0u;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&inbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int sl = 0; sl < 2; sl++) {
        const int b = (sl == 0) ? rank : NBLK - 1 - rank;
        float *sp = slot_ptr(buf, 0, sl);
        for (long long e = threadIdx.x; e < (long long)bs * ldr; e += blockDim.x) {
            const int j = (int)(e / ldr), r = (int)(e % ldr);
            const int c = b * bs + j;
            const bool ok = (c < n && r < n);
            sp[(size_t)j * ldr + r] = ok ? (float)G[r + (long long)c * ldg] : 0.f;
            sp[(size_t)(bs + j) * ldr + r] = (ok && r == c) ? 1.f : 0.f;
        }
    }
    cluster.sync();
    // Block moves: a split cluster barrier instead of a full one per move.  Each thread keeps
    // one arrival outstanding between moves: it arrives once its incoming blocks have landed and
    // waits just before the next move's copies, so every copy of the previous move (which read
    // the buffers the next move writes) is complete, while the wait's latency hides behind the
    // next super-round's Gram, rounds and update.  Sweep ends consume the arrival before their
    // full barriers and re-arm it when another sweep follows.
    cluster_arrive();
    int cur = 0, sweep = 0;
    uint32_t mphase = 0;
    const int nch = ldr / 4;                 // 16-byte row chunks; rows n..ldr-1 are zero
    const uint32_t slot_bytes = (uint32_t)(slot_elems * sizeof(float));
    float wmax = 0.f;                        // warp 0's largest cos^2 and rotations in the sweep
    int wrot = 0;
    for (; sweep < max_sweeps; sweep++) {
        for (int sr = 0; sr < NBLK - 1; sr++) {
            float *s0 = slot_ptr(buf, cur, 0), *s1 = slot_ptr(buf, cur, 1);
            const int b0 = gr_block(rank, 0, sr, NBLK), b1 = gr_block(rank, 1, sr, NBLK);
            auto colw = [&](int c) { return (c < bs) ? s0 + (size_t)c * ldr : s1 + (size_t)(c - bs) * ldr; };
            auto colv = [&](int c) { return (c < bs) ? s0 + (size_t)(bs + c) * ldr : s1 + (size_t)c * ldr; };
            // ---- Gram: partial sums per (block, row slice)
            if (threadIdx.x < KS * NTP) {
                const int bk = threadIdx.x / KS, sl = threadIdx.x - bk * KS;
                int bi = 0, rem = bk;
                while (rem >= NT - bi) { rem -= NT - bi; bi++; }
                const int bj = bi + rem;
                float acc[TK][TK];
#pragma unroll
                for (int a = 0; a < TK; a++)
#pragma unroll
                    for (int c = 0; c < TK; c++) acc[a][c] = 0.f;
                for (int ch = sl; ch < nch; ch += KS) {
                    float4 x[TK], y[TK];
#pragma unroll
                    for (int a = 0; a < TK; a++) x[a] = *reinterpret_cast<const float4 *>(colw(bi * TK + a) + 4 * ch);
#pragma unroll
                    for (int c = 0; c < TK; c++)
                        y[c] = (bi == bj) ? x[c] : *reinterpret_cast<const float4 *>(colw(bj * TK + c) + 4 * ch);
#pragma unroll
                    for (int a = 0; a < TK; a++)
#pragma unroll
                        for (int c = 0; c < TK; c++) {
                            float v = acc[a][c];
                            v = fmaf(x[a].x, y[c].x, v);
                            v = fmaf(x[a].y, y[c].y, v);
                            v = fmaf(x[a].z, y[c].z, v);
                            v = fmaf(x[a].w, y[c].w, v);
                            acc[a][c] = v;
                        }
                }
#pragma unroll
                for (int a = 0; a < TK; a++)
#pragma unroll
                    for (int c = 0; c < TK; c++) red[((bk * TK + a) * TK + c) * KS + sl] = acc[a][c];
            }
            if (threadIdx.x == 0) sr_rot = 0;
            __syncthreads();
            for (int v = threadIdx.x; v < NTP * TK * TK; v += blockDim.x) {
                float sum = 0.f;
#pragma unroll 4
                for (int k = 0; k < KS; k++) sum += red[v * KS + k];
                const int bk = v / (TK * TK), a = (v / TK) % TK, c = v % TK;
                int bi = 0, rem = bk;
                while (rem >= NT - bi) { rem -= NT - bi; bi++; }
                const int i = bi * TK + a, j = (bi + rem) * TK + c;
                gsm[i][j] = sum;
                gsm[j][i] = sum;
            }
            __syncthreads();
            // ---- rounds: Gl on warp 0, Z on warp 1
            if (wid == 0) {
                float g[NL];
                float dg = 0.f;
#pragma unroll
                for (int k = 0; k < NL; k++) {
                    g[k] = lane < NL ? gsm[lane][k] : 0.f;
                    if (k == lane) dg = g[k];
                }
                bool any = false;
                if (sr == 0) gr_rounds_g<BS, true>(g, dg, lane, b0, b1, n, tol, wmax, wrot, any, rot_cs, rot_sn, rot_bal);
                else gr_rounds_g<BS, false>(g, dg, lane, b0, b1, n, tol, wmax, wrot, any, rot_cs, rot_sn, rot_bal);
                if (lane == 0) sr_rot = any ? 1 : 0;
            } else if (wid == 1) {
                float z[NL];
#pragma unroll
                for (int k = 0; k < NL; k++) z[k] = (k == lane) ? 1.f : 0.f;
                if (sr == 0) gr_rounds_z<BS, true>(z, rot_cs, rot_sn, rot_bal);
                else gr_rounds_z<BS, false>(z, rot_cs, rot_sn, rot_bal);
                if (lane < NL) {
#pragma unroll
                    for (int k = 0; k < NL; k++) zsm[lane][k] = z[k];
                }
            }
            __syncthreads();
            // ---- P <- P Z (W and V), one thread per 4-row chunk of one matrix
            if (sr_rot) gr_apply<BS>(s0, s1, ldr, nch, &zsm[0][0]);
            // ---- move blocks to their next holders (positions 1..NBLK-1 rotate by one)
            const int nxt = cur ^ 1;
            int dst0, dsl0, dst1, dsl1;
            if (rank == 0) { dst0 = 0; dsl0 = 0; }
            else if (rank < CLN - 1) { dst0 = rank + 1; dsl0 = 0; }
            else { dst0 = CLN - 1; dsl0 = 1; }
            if (rank == 0) { dst1 = 1; dsl1 = 0; }
            else { dst1 = rank - 1; dsl1 = 1; }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            cluster_wait();                  // the previous move has landed everywhere
            if (threadIdx.x == 0) {
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(&inbar)),
                             "r"(2u * slot_bytes)
                             : "memory");
                for (int sl = 0; sl < 2; sl++) {
                    const int dc = sl ? dst1 : dst0, ds = sl ? dsl1 : dsl0;
                    uint32_t rdst, rbar;
                    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(rdst) : "r"(smem_addr(slot_ptr(buf, nxt, ds))), "r"(dc));
                    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(rbar) : "r"(smem_addr(&inbar)), "r"(dc));
                    asm volatile(
                        "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(rdst),
                        "r"(smem_addr(slot_ptr(buf, cur, sl))), "r"(slot_bytes), "r"(rbar)
                        : "memory");
                }
            }
            {
                uint32_t ok = 0;
                const long long t0 = clock64();
                while (true) {
                    asm volatile(
                        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                        "selp.u32 %0, 1, 0, p;\n\t}\n"
                        : "=r"(ok)
                        : "r"(smem_addr(&inbar)), "r"(mphase)
                        : "memory");
                    if (ok) break;
                    if (clock64() - t0 > (1ll << 31)) { atomicExch(flag, 1); break; }
                }
                mphase ^= 1u;
            }
            cluster_arrive();
            cur = nxt;
        }
        cluster_wait();
        // ---- did any CTA rotate during this sweep, and how large was the largest cosine?
        if (threadIdx.x == 0) {
            sweep_max = __float_as_uint(wmax);
            rot_count = wrot;
        }
        wmax = 0.f;
        wrot = 0;
        __syncthreads();
        if (threadIdx.x < CLN) {
            int *dstf = cluster.map_shared_rank(&sweep_rot[rank], (unsigned)threadIdx.x);
            *dstf = rot_count;
            unsigned int *dstm = cluster.map_shared_rank(&cl_max[rank], (unsigned)threadIdx.x);
            *dstm = sweep_max;
        }
        cluster.sync();
        int total = 0;
        float cmax = 0.f;
#pragma unroll
        for (int c = 0; c < CLN; c++) {
            total += sweep_rot[c];
            cmax = fmaxf(cmax, __uint_as_float(cl_max[c]));
        }
        __syncthreads();
        cluster.sync();
        if (total == 0) break;
        if (cmax < stop_tol) { sweep++; break; }
        if (sweep + 1 < max_sweeps) cluster_arrive();       // the next sweep's first move waits on it
    }
    for (int sl = 0; sl < 2; sl++) {
        float *sp = slot_ptr(buf, cur, sl);
        const int b = gr_block(rank, sl, 0, NBLK);          // a whole sweep of moves restores the start
        for (long long e = threadIdx.x; e < (long long)bs * n; e += blockDim.x) {
            const int j = (int)(e / n), r = (int)(e % n);
            const int c = b * bs + j;
            if (c < n) {
                Wout[r + (long long)c * ldo] = sp[(size_t)j * ldr + r];
                Vout[r + (long long)c * ldo] = sp[(size_t)(bs + j) * ldr + r];
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
// Descending rank of each value (ties by index).  The values are norms (>= +0), whose IEEE bit
// patterns order like the values as 64-bit integers: integer compares, because GB300's FP64
// pipe is a small fraction of its integer rate (FP64 compares made this step ~40 us at n = 272).
// Each block stages all n keys in shared memory (n <= RANK_SMEM_MAX) and ranks its slice.
constexpr int RANK_SMEM_MAX = 6144;
__global__ void rank_desc_kernel(const double *sv, int n, int *rank) {
    extern __shared__ long long s_key[];
    const bool staged = n <= RANK_SMEM_MAX;
    const long long *gkey = reinterpret_cast<const long long *>(sv);
    if (staged) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) s_key[i] = gkey[i];
        __syncthreads();
    }
    const long long *key = staged ? s_key : gkey;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const long long v = key[j];
    int r = 0;
    for (int i = 0; i < n; i++) {
        const long long w = key[i];
        r += (w > v) | ((w == v) & (i < j));
    }
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


// ------------------------------------------------------------------ SVD refinement kernels
// M = I + C, the first-order simultaneous correction of approximate right singular vectors V of X
// (columns v_i; H = (XV)^T (XV), Sm = V^T V, both FP64-accurate, upper triangles read), written as
// its double-float split (Mh + Ml): with h_i = H_ii,
//   C_ii = (1 - Sm_ii) / 2                                  (normalisation),
//   C_ij = (H_ij - Sm_ij (h_i + h_j) / 2) / (h_j - h_i) - Sm_ij / 2    (i != j),
// so that V (I + C) is orthonormal and diagonalises H to second order.  A pair whose correction
// exceeds `tight` (nearly equal h: FP32 could not separate the two vectors, and a first-order
// step applied to many such pairs at once does not converge) gets no coupling term here and is
// listed (key j n + i, i < j; at most max_pairs) for an exact rotation by refine_tight_kernel.
__global__ void refine_update_kernel(const double *H, i64 ldh, const double *Sm, i64 lds, int n, double tight,
                                     float *Mh, float *Ml, i64 ldm, int *pair_count, int *pairs, int max_pairs) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < (i64)n * n; e += (i64)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        double c;
        if (i == j) {
            c = 0.5 * (1.0 - Sm[i + (i64)i * lds]);
        } else {
            const double hi = H[i + (i64)i * ldh], hj = H[j + (i64)j * ldh];
            const int a = min(i, j), b = max(i, j);           // H and Sm hold their upper triangles
            const double hij = H[a + (i64)b * ldh];
            const double sij = Sm[a + (i64)b * lds];
            const double num = hij - sij * 0.5 * (hi + hj);
            const double den = hj - hi;
            if (fabs(num) <= tight * fabs(den)) {
                c = num / den;
            } else {
                c = 0.0;
                if (i < j && num != 0.0) {
                    const int k = atomicAdd(pair_count, 1);
                    if (k < max_pairs) pairs[k] = j * n + i;
                }
            }
            c -= 0.5 * sij;
        }
        const double mv = (i == j ? 1.0 : 0.0) + c;
        const float mh = __double2float_rn(mv);
        Mh[i + (i64)j * ldm] = mh;
        Ml[i + (i64)j * ldm] = __double2float_rn(mv - (double)mh);
    }
}

// Exact FP64 one-sided Jacobi rotations of the listed pairs: for pair (i, j), a = |w_i|^2,
// b = |w_j|^2, d = w_i . w_j over the current columns of W = X V, and (w_i, w_j), (v_i, v_j)
// rotated by the angle that zeroes d (Rutishauser's formulas), so that W = X V still holds
// afterwards.  VW holds V in rows [0, n) and W in rows [n, 2n); its double-float split (hi, lo)
// is rewritten for the rotated columns.  The list (unordered, from refine_update_kernel) is
// sorted (key j n + i ascending) and scheduled into batches of disjoint pairs by first fit in
// that order -- batch(i, j) = 1 + max(batch of the last pair that touched i, ... touched j) --
// so pairs that share a column keep their sorted order and the pairs of a batch are
// independent.  A cluster of TIGHT_CL CTAs runs the batches one after another (a cluster
// barrier between them), one CTA per pair: each rotation is FP64-pipe bound on its SM (~3000
// FP64 operations), so spreading a batch over SMs is what shortens the step.  CTA 0 sorts and
// schedules into `sched` (count, batch offsets, keys by batch); an empty list costs one read.
// Orders above TIGHT_SMEM_N schedule one pair per batch.
constexpr int REFINE_MAX_PAIRS = 2048;
constexpr int TIGHT_CL = 8;
constexpr int TIGHT_SMEM_N = 8192;
__global__ void __cluster_dims__(TIGHT_CL, 1, 1) __launch_bounds__(256)
    refine_tight_kernel(double *VW, i64 ld, float *hi, float *lo, i64 lds, int n, const int *pair_count,
                        const int *pairs, int *sched) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const int crank = (int)cluster.block_rank();
    __shared__ int keys[REFINE_MAX_PAIRS];
    __shared__ unsigned short bat[REFINE_MAX_PAIRS];
    __shared__ int last[TIGHT_SMEM_N];
    __shared__ double red[3][8];
    __shared__ double rot[2];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int cnt = min(*pair_count, REFINE_MAX_PAIRS);
    if (cnt == 0) return;                                  // uniform over the cluster
    int *nbat = sched, *off = sched + 1, *skey = sched + 2 + REFINE_MAX_PAIRS;
    if (crank == 0) {
        int np2 = 1;
        while (np2 < cnt) np2 <<= 1;
        for (int e = tid; e < np2; e += 256) keys[e] = e < cnt ? pairs[e] : INT_MAX;
        for (int e = tid; e < n && e < TIGHT_SMEM_N; e += 256) last[e] = 0;
        __syncthreads();
        for (int k = 2; k <= np2; k <<= 1)
            for (int jj = k >> 1; jj > 0; jj >>= 1) {
                for (int e = tid; e < np2; e += 256) {
                    const int o = e ^ jj;
                    if (o > e) {
                        const bool up = (e & k) == 0;
                        const int a = keys[e], b = keys[o];
                        if ((a > b) == up) { keys[e] = b; keys[o] = a; }
                    }
                }
                __syncthreads();
            }
        if (tid == 0) {
            // first-fit batches in sorted order, then a counting sort of the keys by batch
            int nb = 0;
            for (int q = 0; q < cnt; q++) {
                int b;
                if (n <= TIGHT_SMEM_N) {
                    const int j = keys[q] / n, i = keys[q] - j * n;
                    b = max(last[i], last[j]);
                    last[i] = last[j] = b + 1;
                } else {
                    b = q;
                }
                bat[q] = (unsigned short)b;
                nb = max(nb, b + 1);
            }
            *nbat = nb;
            for (int b = 0; b <= nb; b++) off[b] = 0;
            for (int q = 0; q < cnt; q++) off[bat[q] + 1]++;
            for (int b = 0; b < nb; b++) off[b + 1] += off[b];
            int *fill = last;                      // per-batch fill counters (nb <= cnt <= 2048)
            for (int b = 0; b < nb; b++) fill[b] = 0;
            for (int q = 0; q < cnt; q++) {        // stable: a batch keeps the sorted order
                const int b = bat[q];
                skey[off[b] + fill[b]++] = keys[q];
            }
        }
    }
    cluster.sync();
    const int nb = *nbat;
    for (int b = 0; b < nb; b++) {
        for (int q = off[b] + crank; q < off[b + 1]; q += TIGHT_CL) {
            const int key = skey[q];
            const int j = key / n, p = key - j * n;
            double a = 0.0, bb = 0.0, d = 0.0;
            for (int r = n + tid; r < 2 * n; r += 256) {
                const double x = VW[r + (i64)p * ld], y = VW[r + (i64)j * ld];
                a = fma(x, x, a);
                bb = fma(y, y, bb);
                d = fma(x, y, d);
            }
            a = warp_sum(a);
            bb = warp_sum(bb);
            d = warp_sum(d);
            if (lane == 0) { red[0][wid] = a; red[1][wid] = bb; red[2][wid] = d; }
            __syncthreads();
            if (tid == 0) {
                double A = 0.0, B = 0.0, D = 0.0;
                for (int w = 0; w < 8; w++) { A += red[0][w]; B += red[1][w]; D += red[2][w]; }
                double cs = 1.0, sn = 0.0;
                if (D != 0.0) {
                    const double zeta = (B - A) / (2.0 * D);
                    const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                    cs = 1.0 / sqrt(1.0 + t * t);
                    sn = cs * t;
                }
                rot[0] = cs;
                rot[1] = sn;
            }
            __syncthreads();
            const double cs = rot[0], sn = rot[1];
            for (int r = tid; r < 2 * n; r += 256) {
                const double x = VW[r + (i64)p * ld], y = VW[r + (i64)j * ld];
                const double nx = cs * x - sn * y, ny = sn * x + cs * y;
                VW[r + (i64)p * ld] = nx;
                VW[r + (i64)j * ld] = ny;
                const float hx = __double2float_rn(nx), hy = __double2float_rn(ny);
                hi[r + p * lds] = hx;
                lo[r + p * lds] = __double2float_rn(nx - (double)hx);
                hi[r + j * lds] = hy;
                lo[r + j * lds] = __double2float_rn(ny - (double)hy);
            }
            __syncthreads();
        }
        cluster.sync();
    }
}

// hi = fl32(x), lo = fl32(x - hi), no scaling (entries of order one)
__global__ void split_unit_kernel(const double *x, i64 ld, i64 r, i64 c, float *hi, float *lo, i64 ldo) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < r * c; e += (i64)gridDim.x * blockDim.x) {
        const i64 j = e / r, i = e - j * r;
        const double v = x[i + j * ld];
        const float h = __double2float_rn(v);
        hi[i + j * ldo] = h;
        lo[i + j * ldo] = __double2float_rn(v - (double)h);
    }
}

// xexp[0] <- the split's scale exponent field; the split's own exponent <- 1023 (unit), so that
// products read the scaled matrix X 2^(1023 - xexp) itself
__global__ void take_scale_kernel(int *split_exp, int *xexp) {
    const int e = *split_exp;
    *xexp = e > 0 ? e : 1023;
    *split_exp = 1023;
}

// Column j: sv_j = |w_j| / |v_j| (the Rayleigh quotient of the unnormalised v_j), nrm = (|w_j|, |v_j|).
__global__ void refine_norms_kernel(const double *W, i64 ldw, const double *V, i64 ldv, int n, const int *xexp,
                                    double *sv, double *nrm) {
    const double unscale = ldexp(1.0, *xexp - 1023);
    const int lane = threadIdx.x & 31;
    for (int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); j < n; j += gridDim.x * (blockDim.x >> 5)) {
        double a = 0, b = 0;
        for (int i = lane; i < n; i += 32) {
            const double w = W[i + (i64)j * ldw], v = V[i + (i64)j * ldv];
            a = fma(w, w, a);
            b = fma(v, v, b);
        }
        a = warp_sum(a);
        b = warp_sum(b);
        if (lane == 0) {
            const double nw = sqrt(a), nv = sqrt(b);
            sv[j] = nv > 0.0 ? nw / nv * unscale : 0.0;
            nrm[2 * j] = nw;
            nrm[2 * j + 1] = nv;
        }
    }
}

// U(:, rank j) = w_j / |w_j|, V(:, rank j) = v_j / |v_j|, sv_sorted[rank j] = sv_j
__global__ void refine_scatter_kernel(const double *W, i64 ldw, const double *Vin, i64 ldvi, const double *sv,
                                      const double *nrm, const int *rank, int n, double *U, i64 ldu, double *V,
                                      i64 ldv, double *sv_sorted) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < (i64)n * n; e += (i64)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        const int r = rank[j];
        const double nw = nrm[2 * j], nv = nrm[2 * j + 1];
        U[i + (i64)r * ldu] = nw > 0.0 ? W[i + (i64)j * ldw] / nw : 0.0;
        V[i + (i64)r * ldv] = nv > 0.0 ? Vin[i + (i64)j * ldvi] / nv : 0.0;
        if (i == 0) sv_sorted[r] = sv[j];
    }
}

unsigned gfor(long long n) {
    long long g = (n + 255) / 256;
    return (unsigned)std::max<long long>(1, std::min<long long>(g, (long long)std::max(1, ctx().sms) * 8));
}

}  // namespace

template <typename S>
bool cholesky_small(cudaStream_t s, DM<double> G, double rel_tol, int *d_flag) {
    return chol_factor<S>(s, G, rel_tol, d_flag, nullptr);     // tiled factorisation (k_chol.cu)
}
template bool cholesky_small<double>(cudaStream_t, DM<double>, double, int *);
template bool cholesky_small<float>(cudaStream_t, DM<double>, double, int *);

template <typename S>
int jacobi_small(cudaStream_t s, DM<double> G, DM<double> U, DM<double> V, double *d_sv, int *d_flag,
                 bool want_sweeps) {
    PhaseTimer pt(&ctx().timing.small_ms);
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
    const int ldr = (n + 3) / 4 * 4;
    constexpr int VW = 16 / sizeof(S), MAXIT = sizeof(S) == 4 ? 4 : 8;
    // block-cyclic cluster kernel: 16 CTAs where a non-portable cluster of 16 can be
    // scheduled and each CTA still gets >= 5 columns per slot, else 8
    bool launched = false;
    int variant = 0;                         // cluster size of the block-cyclic kernel that ran
    cudaLaunchAttribute cattr[1];
    cattr[0].id = cudaLaunchAttributeClusterDimension;
    cattr[0].val.clusterDim.x = 8;
    cattr[0].val.clusterDim.y = 1;
    cattr[0].val.clusterDim.z = 1;
    for (int cl : {16, 8}) {
        if (launched || n < 64 || ldr / VW > 32 * MAXIT) break;
        const int nblk = 2 * cl, bs = (n + nblk - 1) / nblk;
        if (cl == 16 && bs < 5) continue;
        if (bs > 32 || 2 * bs > 64) continue;
        const size_t bsmem = sizeof(S) * (size_t)4 * bs * ldr * 2;
        if (bsmem > 200 * 1024) continue;
        // FP32 at the block widths of the common orders (l in (256, 288] on 16 CTAs, l in
        // (96, 112] on 8): the register-resident Gram form
        const bool greg = sizeof(S) == 4 && ((cl == 16 && bs == 9) || (cl == 8 && bs == 7));
        const void *kern = (cl == 16) ? (const void *)jacobi_block_cluster_kernel<S, 16>
                                      : (const void *)jacobi_block_cluster_kernel<S, 8>;
        if (greg) kern = (cl == 16) ? (const void *)jacobi_gramreg_kernel<16, 9> : (const void *)jacobi_gramreg_kernel<8, 7>;
        if (cl == 16 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        RSVD_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bsmem));
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cl);
        cfg.blockDim = dim3(greg ? GR_THREADS : 32 * std::min(bs, 16));
        cfg.dynamicSmemBytes = bsmem;
        cfg.stream = s;
        cattr[0].val.clusterDim.x = cl;
        cfg.attrs = cattr;
        cfg.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) != cudaSuccess || nclusters < 1) {
            cudaGetLastError();
            continue;
        }
        if (greg) {
            if constexpr (sizeof(S) == 4) {
                auto gk = (cl == 16) ? jacobi_gramreg_kernel<16, 9> : jacobi_gramreg_kernel<8, 7>;
                RSVD_CK(cudaLaunchKernelEx(&cfg, gk, (const double *)G.p, (long long)G.ld, n, ldr, (float)tol,
                                           (float)(tol / 10), 40, (float *)W, (float *)Vacc, (long long)ld, d_sweeps,
                                           d_flag));
            }
        } else if (cl == 16) {
            RSVD_CK(cudaLaunchKernelEx(&cfg, jacobi_block_cluster_kernel<S, 16>, (const double *)G.p, (long long)G.ld, n,
                                       bs, ldr, tol, (S)(tol / 10), 40, W, Vacc, (long long)ld, d_sweeps, d_flag));
        } else {
            RSVD_CK(cudaLaunchKernelEx(&cfg, jacobi_block_cluster_kernel<S, 8>, (const double *)G.p, (long long)G.ld, n,
                                       bs, ldr, tol, (S)(tol / 10), 40, W, Vacc, (long long)ld, d_sweeps, d_flag));
        }
        launched = true;
        variant = cl;
    }
    if (!launched && csmem <= 200 * 1024 && n >= 64) {
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
    } else if (!launched) {
        load_kernel_t<S><<<gfor((long long)n * n), 256, 0, s>>>(G.p, G.ld, W, ld, n, 0);
        load_kernel_t<S><<<gfor((long long)n * n), 256, 0, s>>>(G.p, G.ld, Vacc, ld, n, 1);
        jacobi_kernel_t<S><<<1, 1024, 0, s>>>(W, ld, Vacc, ld, n, tol, 40, d_sweeps, d_flag);
    }
    colnorm_kernel_t<S><<<ceil_div(n, 8), 256, 0, s>>>(W, ld, n, d_raw);
    rank_desc_kernel<<<ceil_div(n, 256), 256, n <= RANK_SMEM_MAX ? sizeof(long long) * n : 0, s>>>(d_raw, n, d_rank);
    scatter_kernel_t<S><<<gfor((long long)n * n), 256, 0, s>>>(W, ld, Vacc, ld, d_raw, d_rank, n, U.p, U.ld, V.p, V.ld,
                                                                 d_sv);
    RSVD_LAUNCH_CK();
    ctx().launches += 6;
    // the buffers above are stream-ordered: without a count to report, nothing waits here
    if (!want_sweeps && !ctx().opts.verbose) return 0;
    int sweeps = 0;
    RSVD_CK(cudaMemcpyAsync(&sweeps, d_sweeps, sizeof(int), cudaMemcpyDeviceToHost, s));
    RSVD_CK(cudaStreamSynchronize(s));
    if (ctx().opts.verbose)
        std::fprintf(stderr, "rsvdpack: jacobi n=%d (%s) sweeps=%d cluster=%d\n", n, sizeof(S) == 4 ? "fp32" : "fp64",
                     sweeps, variant);
    return sweeps;
}
template int jacobi_small<double>(cudaStream_t, DM<double>, DM<double>, DM<double>, double *, int *, bool);
template int jacobi_small<float>(cudaStream_t, DM<double>, DM<double>, DM<double>, double *, int *, bool);

// One refinement step: H = W^T W and Sm = V^T V (double-float products), the first-order
// correction [V; W] <- [V; W] (I + C) for every pair of well-separated singular values (W = X V
// is carried along instead of recomputed), and exact FP64 rotations of the flagged
// nearly-equal pairs (refine_tight_kernel).  From the FP32 Jacobi's converged vectors four steps
// (REFINE_STEPS) bring the singular values to ~1e-15 relative (a step roughly squares the error of
// the separated pairs; nearly-equal pairs, which FP32 cannot separate, are settled by the
// rotations in the first steps).  X is scaled once by a power of two (its largest entry into [1, 2)), so that every
// operand has entries of order one and is split without a scale; the products write the split of
// their result for the next product.
void svd_refine(cudaStream_t s, DM<double> X, DM<double> V, DM<double> U, double *d_sv, int steps) {
    const int n = (int)X.r;
    if (X.r != X.c || V.r != n || V.c != n || U.r != n || U.c != n) fail(RSVD_ERR_ARGUMENT, "svd_refine: shapes");
    if (n == 0) return;
    DBuf xe_b(sizeof(int) * (1 + steps), s), pair_b(sizeof(int) * REFINE_MAX_PAIRS, s),
        sched_b(sizeof(int) * (2 + 2 * (size_t)REFINE_MAX_PAIRS), s);
    int *xexp = (int *)xe_b.get(), *pair_count = xexp + 1;      // one pair counter per step
    int *pairs = (int *)pair_b.get(), *sched = (int *)sched_b.get();
    RSVD_CK(cudaMemsetAsync(pair_count, 0, sizeof(int) * steps, s));
    Df64Split Xs(s, X);
    take_scale_kernel<<<1, 1, 0, s>>>(Xs.exp, xexp);
    RSVD_LAUNCH_CK();
    const i64 ldvw = pad_ld(2 * (i64)n);
    // [V; W] stacks (2n x n, FP64) and their splits, ping-pong
    DMat<double> VWa(2 * n, n, s, false), VWb(2 * n, n, s, false), H(n, n, s, false), Sm(n, n, s, false);
    DBuf sa(sizeof(float) * 2 * (size_t)(ldvw * n), s), sb(sizeof(float) * 2 * (size_t)(ldvw * n), s),
        sm(sizeof(float) * 2 * (size_t)(pad_ld(n) * n), s);
    float *ha = (float *)sa.get(), *la = ha + ldvw * n, *hb = (float *)sb.get(), *lb = hb + ldvw * n;
    float *hm = (float *)sm.get(), *lm = hm + pad_ld(n) * n;
    const int *unit = Xs.exp;                         // 1023 after take_scale_kernel
    RSVD_CK(cudaMemcpy2DAsync(VWa.v.p, sizeof(double) * VWa.v.ld, V.p, sizeof(double) * V.ld, sizeof(double) * n, n,
                              cudaMemcpyDeviceToDevice, s));
    split_unit_kernel<<<gfor((long long)n * n), 256, 0, s>>>(VWa.v.p, VWa.v.ld, n, n, ha, la, ldvw);
    RSVD_LAUNCH_CK();
    {
        const Df64View Vv{ha, la, n, n, ldvw, unit};
        const Df64Out wo{ha + n, la + n, ldvw};
        df64_gemm(s, false, false, 1.0, Xs.view(), Vv, 0.0, VWa.v.sub(n, 0, n, n), &wo);      // W = X V
    }
    DM<double> cur = VWa.v, nxt = VWb.v;
    float *ch = ha, *cl = la, *nh = hb, *nl = lb;
    for (int it = 0; it < steps; it++) {
        const Df64View VWv{ch, cl, 2 * (i64)n, n, ldvw, unit};
        const Df64View Vv = VWv.rows(0, n), Wv = VWv.rows(n, n);
        df64_gram_pair(s, Wv, H.v, Vv, Sm.v);                                   // H = W^T W, Sm = V^T V
        // the last step also settles pairs still coupled beyond 2e-5 by exact rotations, so that
        // the first-order step leaves nearly equal singular values' vectors orthogonal to
        // ~(2e-5)^2 whatever the FP32 Jacobi's last sweep left
        const double tight = (it == steps - 1) ? 2e-5 : 0.005;
        refine_update_kernel<<<gfor((long long)n * n), 256, 0, s>>>(H.v.p, H.v.ld, Sm.v.p, Sm.v.ld, n, tight, hm, lm,
                                                                     pad_ld(n), pair_count + it, pairs,
                                                                     REFINE_MAX_PAIRS);
        RSVD_LAUNCH_CK();
        const Df64View Mv{hm, lm, n, n, pad_ld(n), unit};
        const Df64Out no{nh, nl, ldvw};
        df64_gemm(s, false, false, 1.0, VWv, Mv, 0.0, nxt, &no);                  // [V; W] (I + C)
        refine_tight_kernel<<<TIGHT_CL, 256, 0, s>>>(nxt.p, nxt.ld, nh, nl, ldvw, n, pair_count + it, pairs, sched);
        RSVD_LAUNCH_CK();
        std::swap(cur, nxt);
        std::swap(ch, nh);
        std::swap(cl, nl);
    }
    DBuf nb(sizeof(double) * 3 * (size_t)n, s), rb(sizeof(int) * (size_t)n, s);
    double *raw = (double *)nb.get(), *nrm = raw + n;
    int *rank = (int *)rb.get();
    const double *Wp = cur.p + n, *Vp = cur.p;
    refine_norms_kernel<<<ceil_div(n, 8), 256, 0, s>>>(Wp, cur.ld, Vp, cur.ld, n, xexp, raw, nrm);
    rank_desc_kernel<<<ceil_div(n, 256), 256, n <= RANK_SMEM_MAX ? sizeof(long long) * n : 0, s>>>(raw, n, rank);
    refine_scatter_kernel<<<gfor((long long)n * n), 256, 0, s>>>(Wp, cur.ld, Vp, cur.ld, raw, nrm, rank, n, U.p,
                                                                  U.ld, V.p, V.ld, d_sv);
    RSVD_LAUNCH_CK();
    ctx().launches += 6 + 3 * steps;
    if (ctx().opts.verbose) {
        std::vector<int> cnt((size_t)steps);
        RSVD_CK(cudaMemcpyAsync(cnt.data(), pair_count, sizeof(int) * steps, cudaMemcpyDeviceToHost, s));
        RSVD_CK(cudaStreamSynchronize(s));
        std::fprintf(stderr, "rsvdpack: refine n=%d tight pairs per step:", n);
        for (int c : cnt) std::fprintf(stderr, " %d", c);
        std::fprintf(stderr, "\n");
    }
}

void small_svd_refined(cudaStream_t s, DM<double> G, DM<double> U, DM<double> V, double *d_sv, int *d_flag) {
    jacobi_small<float>(s, G, U, V, d_sv, d_flag, false);
    PhaseTimer pt(&ctx().timing.small_ms);
    svd_refine(s, G, V, U, d_sv, REFINE_STEPS);
}

}  // namespace rsvd
