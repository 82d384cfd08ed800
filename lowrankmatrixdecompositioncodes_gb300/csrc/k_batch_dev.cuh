// k_batch_dev.cuh -- the batched rSVD's persistent kernel (see k_batch.cu for the pipeline),
// included by one k_batch_lp*.cu file per instantiation.
#pragma once
#include "k_batch.h"
#include "k_common.cuh"

#include <cmath>

namespace rsvd {

namespace {


struct U4b { uint32_t x, y, z, w; };
__device__ __forceinline__ U4b philox_b(U4b c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = U4b{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// Om (n x l, column-major element e = row + col*n) into shared memory, row-major Bsm[j*l + c].
// Same counter layout as the single-matrix generator: group g = e/4 -> counter (g, offset).
__device__ void gen_omega(float *Bsm, int n, int l, uint64_t seed, uint64_t offset) {
    const long long total = (long long)n * l, groups = (total + 3) / 4;
    for (long long g = threadIdx.x; g < groups; g += blockDim.x) {
        const U4b v = philox_b(U4b{(uint32_t)g, (uint32_t)(g >> 32), (uint32_t)offset, (uint32_t)(offset >> 32)},
                               (uint32_t)seed, (uint32_t)(seed >> 32));
        const uint32_t u[4] = {v.x, v.y, v.z, v.w};
        float z[4];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const float u1 = ((float)u[2 * h] + 1.0f) * 2.3283064365386963e-10f;
            const float u2 = (float)u[2 * h + 1] * 2.3283064365386963e-10f;
            const float rad = sqrtf(-2.0f * logf(u1));
            float sn, cs;
            sincospif(2.0f * u2, &sn, &cs);
            z[2 * h] = rad * cs;
            z[2 * h + 1] = rad * sn;
        }
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const long long e = 4 * g + t;
            if (e < total) {
                const int row = (int)(e % n), col = (int)(e / n);
                Bsm[(size_t)row * l + col] = z[t];
            }
        }
    }
}

// Register tiles of the two per-item products: thread t owns 4 consecutive rows (t / 16)
// and the columns c = t % 16 + 16 u, u < 5 (l <= 80), so that one 16-byte load of A and five
// broadcast loads of B feed 20 FMAs; the next chunk of A is prefetched into registers while
// the current one is multiplied.
constexpr int CU_MAX = 5;        // column groups per thread: l <= 16 * CU_MAX
// The products are instantiated for CU = 1..5 column groups and each call takes the
// smallest CU with 16 * CU >= its width (l, or k for the output products): at the batch's
// mean width (~37) the fixed CU = 5 spent 40% of its FMAs on zero padding.

// Y (m x l, ldy) = A (m x n) * B, B row-major in shared memory (B[j*l + c]).
// Row tiles of 64; A chunks of 64 rows x 32 columns staged as At[jj][row] (pitch ATP).
template <int CU>
__device__ void gemm_A_B_t(const float *A, long long lda, int m, int n, const float *Bsm, int l, float *Y,
                           long long ldy, float *At) {
    const int tid = threadIdx.x, rg = (tid >> 4) * 4, cg = tid & 15;
    for (int r0 = 0; r0 < m; r0 += 64) {
        float acc[4][CU];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int u = 0; u < CU; u++) acc[a][u] = 0.f;
        float pre[8];
        auto fetch = [&](int j0) {
#pragma unroll
            for (int t = 0; t < 8; t++) {
                const int e = tid + BT * t, rr = e & 63, jj = e >> 6;
                pre[t] = (r0 + rr < m && j0 + jj < n) ? A[(r0 + rr) + (long long)(j0 + jj) * lda] : 0.f;
            }
        };
        fetch(0);
        for (int j0 = 0; j0 < n; j0 += 32) {
            __syncthreads();
#pragma unroll
            for (int t = 0; t < 8; t++) {
                const int e = tid + BT * t;
                At[(e >> 6) * ATP + (e & 63)] = pre[t];
            }
            __syncthreads();
            if (j0 + 32 < n) fetch(j0 + 32);
            const int jn = min(32, n - j0);
            for (int jj = 0; jj < jn; jj++) {
                const float4 a4 = *reinterpret_cast<const float4 *>(At + jj * ATP + rg);
                const float av[4] = {a4.x, a4.y, a4.z, a4.w};
                const float *b = Bsm + (size_t)(j0 + jj) * l;
                float bv[CU];
#pragma unroll
                for (int u = 0; u < CU; u++) {
                    const int c = cg + 16 * u;
                    bv[u] = (c < l) ? b[c] : 0.f;
                }
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int u = 0; u < CU; u++) acc[a][u] = fmaf(av[a], bv[u], acc[a][u]);
            }
        }
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const int r = r0 + rg + a;
            if (r < m) {
#pragma unroll
                for (int u = 0; u < CU; u++) {
                    const int c = cg + 16 * u;
                    if (c < l) Y[r + (long long)c * ldy] = acc[a][u];
                }
            }
        }
    }
    __syncthreads();
}

// Z (n x l, ldz) = A^T (n x m) * Q (m x l, ldq, global).  Column tiles of 64 (thread: 4
// columns of A); row chunks of 32 staged as At[ii][col] (pitch ATP) and Qs[ii][c].
template <int CU>
__device__ void gemm_At_Q_t(const float *A, long long lda, int m, int n, const float *Q, long long ldq, int l,
                            float *Z, long long ldz, float *At, float *Qs) {
    const int tid = threadIdx.x, jg = (tid >> 4) * 4, cg = tid & 15;
    for (int j0 = 0; j0 < n; j0 += 64) {
        float acc[4][CU];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int u = 0; u < CU; u++) acc[a][u] = 0.f;
        float pa[8], pq[2 * CU];          // Q: 32 rows x 16 CU columns over BT threads
        auto fetch = [&](int i0) {
#pragma unroll
            for (int t = 0; t < 8; t++) {
                const int e = tid + BT * t, ii = e & 31, jj = e >> 5;
                pa[t] = (i0 + ii < m && j0 + jj < n) ? A[(i0 + ii) + (long long)(j0 + jj) * lda] : 0.f;
            }
#pragma unroll
            for (int t = 0; t < 2 * CU; t++) {
                const int e = tid + BT * t, ii = e & 31, c = e >> 5;
                pq[t] = (c < l && i0 + ii < m) ? Q[(i0 + ii) + (long long)c * ldq] : 0.f;
            }
        };
        fetch(0);
        for (int i0 = 0; i0 < m; i0 += 32) {
            __syncthreads();
#pragma unroll
            for (int t = 0; t < 8; t++) {
                const int e = tid + BT * t;
                At[(e & 31) * ATP + (e >> 5)] = pa[t];
            }
#pragma unroll
            for (int t = 0; t < 2 * CU; t++) {
                const int e = tid + BT * t, c = e >> 5;
                if (c < l) Qs[(e & 31) * l + c] = pq[t];
            }
            __syncthreads();
            if (i0 + 32 < m) fetch(i0 + 32);
            const int in = min(32, m - i0);
            for (int ii = 0; ii < in; ii++) {
                const float4 a4 = *reinterpret_cast<const float4 *>(At + ii * ATP + jg);
                const float av[4] = {a4.x, a4.y, a4.z, a4.w};
                const float *qr = Qs + ii * l;
                float bv[CU];
#pragma unroll
                for (int u = 0; u < CU; u++) {
                    const int c = cg + 16 * u;
                    bv[u] = (c < l) ? qr[c] : 0.f;
                }
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int u = 0; u < CU; u++) acc[a][u] = fmaf(av[a], bv[u], acc[a][u]);
            }
        }
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const int j = j0 + jg + a;
            if (j < n) {
#pragma unroll
                for (int u = 0; u < CU; u++) {
                    const int c = cg + 16 * u;
                    if (c < l) Z[j + (long long)c * ldz] = acc[a][u];
                }
            }
        }
    }
    __syncthreads();
}

// The column-group count of a product: the smallest that covers its width, plus the tuned
// offset cuadd (0 or 1: one more group leaves padding FMAs but fewer loop trips per row chunk).
__device__ __forceinline__ int cu_for(int l, int cuadd) { return min(CU_MAX, (l + 15) / 16 + cuadd); }

__device__ __forceinline__ void gemm_A_B(const float *A, long long lda, int m, int n, const float *Bsm, int l,
                                         float *Y, long long ldy, float *At, int cuadd) {
    switch (cu_for(l, cuadd)) {
        case 1: gemm_A_B_t<1>(A, lda, m, n, Bsm, l, Y, ldy, At); break;
        case 2: gemm_A_B_t<2>(A, lda, m, n, Bsm, l, Y, ldy, At); break;
        case 3: gemm_A_B_t<3>(A, lda, m, n, Bsm, l, Y, ldy, At); break;
        case 4: gemm_A_B_t<4>(A, lda, m, n, Bsm, l, Y, ldy, At); break;
        default: gemm_A_B_t<CU_MAX>(A, lda, m, n, Bsm, l, Y, ldy, At); break;
    }
}
__device__ __forceinline__ void gemm_At_Q(const float *A, long long lda, int m, int n, const float *Q, long long ldq,
                                          int l, float *Z, long long ldz, float *At, float *Qs, int cuadd) {
    switch (cu_for(l, cuadd)) {
        case 1: gemm_At_Q_t<1>(A, lda, m, n, Q, ldq, l, Z, ldz, At, Qs); break;
        case 2: gemm_At_Q_t<2>(A, lda, m, n, Q, ldq, l, Z, ldz, At, Qs); break;
        case 3: gemm_At_Q_t<3>(A, lda, m, n, Q, ldq, l, Z, ldz, At, Qs); break;
        case 4: gemm_At_Q_t<4>(A, lda, m, n, Q, ldq, l, Z, ldz, At, Qs); break;
        default: gemm_At_Q_t<CU_MAX>(A, lda, m, n, Q, ldq, l, Z, ldz, At, Qs); break;
    }
}

// G (l x l, shared, ldg = l) = Y^T Y for Y (rows x l) in global; 32-row chunks staged.
__device__ void gram_cta(const float *Y, long long ldy, int rows, int l, float *G, float *Ys) {
    // upper 4 x 4 tiles of G, one per thread (l <= 80: at most 210 tiles); 32-row chunks of Y
    // staged row-major (Ys[row * LP + col]) so a tile row is two 16-byte loads for 16 FMAs
    const int tid = threadIdx.x;
    const int ng = (l + 3) / 4, LP = 4 * ng;
    const int ntile = ng * (ng + 1) / 2;
    const bool act = tid < ntile;
    int gj = 0;
    if (act)
        while ((gj + 1) * (gj + 2) / 2 <= tid) gj++;
    const int gi = act ? tid - gj * (gj + 1) / 2 : 0;
    float acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[a][c] = 0.f;
    for (int r0 = 0; r0 < rows; r0 += 32) {
        __syncthreads();
        for (int e = tid; e < 32 * LP; e += BT) {
            const int rr = e & 31, c = e >> 5;
            Ys[rr * LP + c] = (r0 + rr < rows && c < l) ? Y[(r0 + rr) + (long long)c * ldy] : 0.f;
        }
        __syncthreads();
        if (act) {
            const int rn = min(32, rows - r0);
            for (int rr = 0; rr < rn; rr++) {
                const float4 x4 = *reinterpret_cast<const float4 *>(Ys + rr * LP + 4 * gi);
                const float4 y4 = *reinterpret_cast<const float4 *>(Ys + rr * LP + 4 * gj);
                const float xv[4] = {x4.x, x4.y, x4.z, x4.w}, yv[4] = {y4.x, y4.y, y4.z, y4.w};
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int c = 0; c < 4; c++) acc[a][c] = fmaf(xv[a], yv[c], acc[a][c]);
            }
        }
    }
    if (act) {
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const int i = 4 * gi + a, j = 4 * gj + c;
                if (i < l && j < l) {
                    G[i + j * l] = acc[a][c];
                    G[j + i * l] = acc[a][c];
                }
            }
    }
    __syncthreads();
}

// In-place upper Cholesky of G (l x l, shared); returns false on breakdown (CTA-uniform).
__device__ bool chol_cta(float *G, int l, int *bad) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) *bad = 0;
    __syncthreads();
    for (int j = 0; j < l; j++) {
        if (tid == 0) {
            const float d = G[j + j * l];
            if (!(d > 0.f) || !isfinite(d)) { *bad = 1; G[j + j * l] = 1.f; }
            else G[j + j * l] = sqrtf(d);
        }
        __syncthreads();
        const float p = G[j + j * l];
        for (int k = j + 1 + tid; k < l; k += BT) G[j + k * l] /= p;
        __syncthreads();
        for (int k = j + 1 + wid; k < l; k += BT / 32) {
            const float rjk = G[j + k * l];
            for (int i = j + 1 + lane; i <= k; i += 32) G[i + k * l] -= G[j + i * l] * rjk;
        }
        __syncthreads();
    }
    for (int e = tid; e < l * l; e += BT) {
        const int i = e % l, k = e / l;
        if (i > k) G[e] = 0.f;
    }
    __syncthreads();
    return *bad == 0;
}

// X = R^-1 (upper, l x l, shared, stored row-major: X[j * l + c]), one warp per column.
__device__ void trinv_cta(const float *R, int l, float *X) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int e = threadIdx.x; e < l * l; e += BT) X[e] = 0.f;
    __syncthreads();
    for (int c = wid; c < l; c += BT / 32) {
        float b[3];   // rows lane, lane+32, lane+64 (l <= 96)
#pragma unroll
        for (int t = 0; t < 3; t++) b[t] = (lane + 32 * t == c) ? 1.f : 0.f;
        for (int j = c; j >= 0; j--) {
            const int slot = j >> 5, owner = j & 31;
            float bj = (slot == 0) ? b[0] : (slot == 1 ? b[1] : b[2]);
            bj = __shfl_sync(0xffffffffu, bj, owner);
            const float xj = bj / R[j + j * l];
            if (lane == 0) X[j * l + c] = xj;                        // row-major: the B operand of the product
#pragma unroll
            for (int t = 0; t < 3; t++) {
                const int r = lane + 32 * t;
                if (r < j) b[t] -= xj * R[r + j * l];
            }
        }
    }
    __syncthreads();
}

// CholeskyQR (passes 1 or 2) of Y (rows x l, global) in place; R (shared l x l) = R2 R1.
// A pass whose Cholesky breaks down (Y too ill-conditioned for an FP32 Gram) is redone as
// shifted CholeskyQR: the Gram's diagonal is raised by 8 l u trace(G), which keeps it
// positive definite, and one extra plain pass restores the orthogonality (shifted
// CholeskyQR3, Fukaya et al. 2020).
// Y <- Y R^-1 is the tiled product gemm_A_B applied in place (each 64-row tile of Y is read
// completely before it is written), with R^-1 row-major in X.
__device__ bool cqr_cta(float *Y, long long ldy, int rows, int l, int passes, float *R, float *G, float *X, float *T,
                        float *Ys, float *At, int *bad, int cuadd) {
    for (int e = threadIdx.x; e < l * l; e += BT) R[e] = ((e % l) == (e / l)) ? 1.f : 0.f;
    __syncthreads();
    __shared__ float trace_sh;
    int shifted = 0;
    for (int pass = 0; pass < passes; pass++) {
        gram_cta(Y, ldy, rows, l, G, Ys);
        for (int e = threadIdx.x; e < l * l; e += BT) T[e] = G[e];
        __syncthreads();
        if (!chol_cta(G, l, bad)) {
            if (shifted) return false;
            if (threadIdx.x == 0) {
                float tr = 0.f;
                for (int j = 0; j < l; j++) tr += T[j + j * l];
                trace_sh = tr;
            }
            __syncthreads();
            const float shift = 8.f * (float)l * 1.1920929e-7f * trace_sh;
            for (int e = threadIdx.x; e < l * l; e += BT) G[e] = T[e] + (((e % l) == (e / l)) ? shift : 0.f);
            __syncthreads();
            if (!chol_cta(G, l, bad)) return false;
            shifted = 1;
            passes++;
        }
        trinv_cta(G, l, X);
        gemm_A_B(Y, ldy, rows, l, X, l, Y, ldy, At, cuadd);
        // R <- G R  (both upper)
        for (int e = threadIdx.x; e < l * l; e += BT) {
            const int i = e % l, k = e / l;
            float s = 0.f;
            for (int t = i; t <= k; t++) s = fmaf(G[i + t * l], R[t + k * l], s);
            T[e] = (i <= k) ? s : 0.f;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < l * l; e += BT) R[e] = T[e];
        __syncthreads();
    }
    return true;
}

// One-sided Jacobi on W (l x l, shared), V accumulated; then sort descending.
template <int LP>
__device__ int jacobi_cta(float *W, float *V, int l, float *sv, int *rot) {
    // one-sided Jacobi, round-robin pairs; each pair is handled by a group of LP lanes (4, 8, 16
    // or 32: BT / LP groups per CTA; with LP = 8, every pair of a round (l / 2 <= 36) runs at once
    // for l <= 64; LP = 32 is one warp per pair)
    const int tid = threadIdx.x, g8 = tid / LP, gl = tid % LP;
    const unsigned gmask = (LP == 32) ? 0xffffffffu : (((1u << LP) - 1u) << (tid & (32 - LP)));
    for (int e = tid; e < l * l; e += BT) V[e] = ((e % l) == (e / l)) ? 1.f : 0.f;
    const int np = l + (l & 1);
    const float tol = 4.f * sqrtf((float)l) * 1.1920929e-7f;
    int sweep = 0;
    for (; sweep < 40; sweep++) {
        if (tid == 0) *rot = 0;
        __syncthreads();
        for (int r = 0; r < np - 1; r++) {
            for (int pi = g8; pi < np / 2; pi += BT / LP) {
                int p, q;
                const int mm = np - 1;
                if (pi == 0) { p = 0; q = (r % mm) + 1; }
                else { p = ((r + pi) % mm) + 1; q = ((r - pi + mm) % mm) + 1; }
                const bool valid = (p < l && q < l);
                if (p > q) { const int t = p; p = q; q = t; }
                float a = 0, b = 0, d = 0;
                float *wp = W + p * l, *wq = W + q * l;
                if (valid)
                    for (int i = gl; i < l; i += LP) {
                        const float x = wp[i], y = wq[i];
                        a = fmaf(x, x, a); b = fmaf(y, y, b); d = fmaf(x, y, d);
                    }
#pragma unroll
                for (int o = LP / 2; o > 0; o >>= 1) {
                    a += __shfl_xor_sync(gmask, a, o);
                    b += __shfl_xor_sync(gmask, b, o);
                    d += __shfl_xor_sync(gmask, d, o);
                }
                if (!valid || d == 0.f || fabsf(d) <= tol * sqrtf(a * b)) continue;
                const float zeta = (b - a) / (2.f * d);
                const float t = copysignf(1.f, zeta) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
                const float cs = rsqrtf(1.f + t * t), sn = cs * t;
                float *vp = V + p * l, *vq = V + q * l;
                for (int i = gl; i < l; i += LP) {
                    const float x = wp[i], y = wq[i];
                    wp[i] = cs * x - sn * y;
                    wq[i] = sn * x + cs * y;
                    const float u = vp[i], v = vq[i];
                    vp[i] = cs * u - sn * v;
                    vq[i] = sn * u + cs * v;
                }
                if (gl == 0) *rot = 1;
            }
            __syncthreads();
        }
        const int any = *rot;
        __syncthreads();
        if (!any) break;
    }
    const int lane = tid & 31, wid = tid >> 5;
    for (int c = wid; c < l; c += BT / 32) {
        float s2 = 0.f;
        for (int i = lane; i < l; i += 32) s2 = fmaf(W[i + c * l], W[i + c * l], s2);
        s2 = warp_sum(s2);
        if (lane == 0) sv[c] = sqrtf(s2);
    }
    __syncthreads();
    return sweep;
}


template <int LP>
__global__ void __launch_bounds__(BT, 1)
    batch_rsvd_kernel(const BatchItem *items, int count, int *queue, float *work, long long slab, long long ldw,
                      uint64_t seed, int q, int s, int *flag, int cuadd) {
    extern __shared__ __align__(16) float sm[];
    __shared__ int item_idx, bad, rot;
    float *slabp = work + (long long)blockIdx.x * slab;
    float *Yg = slabp, *Zg = slabp + ldw * 96;   // two tall buffers (<= 96 columns each), ld = ldw
    for (;;) {
        if (threadIdx.x == 0) item_idx = atomicAdd(queue, 1);
        __syncthreads();
        const int it = item_idx;
        __syncthreads();
        if (it >= count) break;
        const BatchItem B = items[it];
        const int m = B.m, n = B.n, l = B.l, k = B.k;
        // shared layout: [Bsm: n*l][At: 64*32]  (phase 1)  /  small l x l work areas (later)
        float *Bsm = sm, *At = sm + ((size_t)n * l + 3) / 4 * 4;        // At: 16-byte aligned
        gen_omega(Bsm, n, l, seed, (uint64_t)B.index);
        __syncthreads();
        gemm_A_B(B.A, B.lda, m, n, Bsm, l, Yg, ldw, At, cuadd);
        // small-matrix areas after the phase-1 region is no longer needed
        const int L2 = l * l;
        float *R = sm, *G = R + L2, *X = G + L2, *T = X + L2, *Ys = T + L2, *W = Ys + 33 * 96, *Vs = W + L2;
        float *sv = Vs + L2, *Qs = sv + 96;
        float *At2 = sm + ((size_t)(Qs + 32 * 96 - sm) + 3) / 4 * 4;   // A chunks of the A^T Q product
        bool ok = true;
        for (int j = 1; j < q && ok; j++) {                            // q-1 power rounds, s=1 schedule
            if ((2 * j - 2) % s == 0) ok = cqr_cta(Yg, ldw, m, l, 1, R, G, X, T, Ys, At2, &bad, cuadd);
            gemm_At_Q(B.A, B.lda, m, n, Yg, ldw, l, Zg, ldw, At2, Qs, cuadd);
            if ((2 * j - 1) % s == 0 && ok) ok = cqr_cta(Zg, ldw, n, l, 1, R, G, X, T, Ys, At2, &bad, cuadd);
            // Y = A Zo : stage Zo row-major in shared memory as the B operand
            for (int e = threadIdx.x; e < n * l; e += BT) Bsm[(e % n) * l + e / n] = Zg[(e % n) + (long long)(e / n) * ldw];
            __syncthreads();
            gemm_A_B(B.A, B.lda, m, n, Bsm, l, Yg, ldw, At, cuadd);
        }
        if (ok) ok = cqr_cta(Yg, ldw, m, l, 2, R, G, X, T, Ys, At2, &bad, cuadd);                // Q in Yg
        if (ok) gemm_At_Q(B.A, B.lda, m, n, Yg, ldw, l, Zg, ldw, At2, Qs, cuadd);  // Bt in Zg
        if (ok) ok = cqr_cta(Zg, ldw, n, l, 2, R, G, X, T, Ys, At2, &bad, cuadd);                // Qh in Zg, Rh in R
        if (!ok) {
            if (threadIdx.x == 0) atomicAdd(flag, 1);
            continue;
        }
        // Jacobi on Rh^T (rows of the triangular factor of a graded matrix are nearly
        // orthogonal, so fewer sweeps): Rh^T = W diag(1/sv) ... i.e. Rh = Vs S (W / sv)^T
        for (int e = threadIdx.x; e < L2; e += BT) W[e] = R[(e / l) + (e % l) * l];
        __syncthreads();
        jacobi_cta<LP>(W, Vs, l, sv, &rot);
        // order: rank of each column by descending sv
        __shared__ int rank_of[96];
        for (int c = threadIdx.x; c < l; c += BT) {
            int r = 0;
            for (int t = 0; t < l; t++) r += (sv[t] > sv[c]) || (sv[t] == sv[c] && t < c);
            rank_of[c] = r;
        }
        __syncthreads();
        // Rh = Uh S Vh^T with Uh = Vs, Vh = W / sv.  U = Q Vh(:, :k) ; V = Qh Uh(:, :k).
        // The k selected columns (by rank) go row-major into T (Vh) and G (Uh), the B operands
        // of the tiled product (rows t, columns r: B[t * k + r]).
        for (int e = threadIdx.x; e < L2; e += BT) {
            const int i = e % l, c = e / l, r = rank_of[c];
            if (r < k) {
                T[i * k + r] = (sv[c] > 0.f) ? W[i + c * l] / sv[c] : 0.f;
                G[i * k + r] = Vs[i + c * l];
            }
        }
        for (int c = threadIdx.x; c < l; c += BT)
            if (rank_of[c] < k) B.S[rank_of[c]] = (double)sv[c];
        __syncthreads();
        gemm_A_B(Yg, ldw, m, l, T, k, B.U, B.ldu, At2, cuadd);
        gemm_A_B(Zg, ldw, n, l, G, k, B.V, B.ldv, At2, cuadd);
        __syncthreads();
    }
}


template <int LP>
void batch_rsvd_launch_impl(cudaStream_t s, const BatchItem *d_items, int count, int *d_queue, float *d_work,
                            long long slab, long long ldw, unsigned long long seed, int q, int s_, int *d_flag,
                            int nctas, size_t smem, int cuadd) {
    auto k = batch_rsvd_kernel<LP>;
    RSVD_CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<nctas, BT, smem, s>>>(d_items, count, d_queue, d_work, slab, ldw, seed, q, s_, d_flag, cuadd);
    RSVD_LAUNCH_CK();
}

}  // namespace

}  // namespace rsvd
