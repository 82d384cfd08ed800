// k_df64.cu -- FP64-accurate matrix products computed on the FP32 pipe ("double-float" GEMM).
//
// GB300 executes FP64 at ~2 FMA/clock/SM and FP32 at 128, so an FP64 product is built here from
// FP32 parts.  Each FP64 operand element x is split once (df64_split) into x = hi + lo with
// hi = x rounded to FP32 and lo = x - hi rounded to FP32 (|x - hi - lo| <= 2^-48 |x|).  The
// product a b is taken as
//   hi_a hi_b   exactly, as p + e with p = fl(hi_a hi_b) and e = fma(hi_a, hi_b, -p)
//               (Dekker's two-product with a fused multiply-add),
//   + hi_a lo_b + lo_a hi_b   in FP32 (their rounding is ~2^-48 |ab|; lo_a lo_b is dropped).
// The running sum of the p's is a compensated pair (s, c): Knuth's two-sum t = s + p,
// z = t - s, err = (s - (t - z)) + (p - z) is exact, s <- t and c <- c + err; the e's and the
// cross terms accumulate into c.  Every four terms the pair is renormalised (s, c) <- two-sum
// (s, c) so that |c| stays below ~2^-23 |s| and c's own roundings stay ~2^-47 |s| each (left to
// grow, c reaches ~sqrt(K) 2^-24 |s| and its roundings add up to ~K 2^-47 |s|).  The result s + c
// is formed in FP64.  This is the
// double-float arithmetic of Dekker (1971) and Knuth (TAOCP vol. 2, 4.2.2) as used for GPUs by
// Thall (2006) and in the QD library (Hida, Li, Bailey 2001).  Accuracy: ~2^-47 relative per
// product term and accumulation step (FP64 gives 2^-53), growing like sqrt(K) for random
// rounding; cost: ~13.5 FP32 operations per multiply-add, ~4x the rate of the FP64 pipe on GB300.
//
// Range: hi and lo are FP32, so the operands are scaled by a power of two chosen on the device
// (df64_split: the largest |x| is brought to [1, 2)), which is exact and is undone in FP64 on
// the result.  Elements below 2^-126 of the largest one lose relative accuracy (their
// contribution to any product is below the accuracy stated above).
#include "rsvd_internal.h"
#include "k_common.cuh"

#include <algorithm>
#include <cmath>

namespace rsvd {

namespace {

// ------------------------------------------------------------------ split with device-side scale
// scale_exp[0] receives the binary exponent E of the largest |x| (0 for an all-zero matrix);
// the split parts are x * 2^-E.
__global__ void maxexp_kernel(const double *x, i64 ld, i64 r, i64 c, int *scale_exp) {
    unsigned long long mx = 0;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < r * c; e += (i64)gridDim.x * blockDim.x) {
        const i64 j = e / r, i = e - j * r;
        const unsigned long long b = (unsigned long long)__double_as_longlong(x[i + j * ld]) & 0x7fffffffffffffffull;
        mx = b > mx ? b : mx;           // |x| orders like its bit pattern
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = y > mx ? y : mx;
    }
    __shared__ unsigned long long wmax[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) wmax[wid] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) mx = wmax[w] > mx ? wmax[w] : mx;
        // exponent field of the largest finite |x| (encoded so that larger means larger)
        atomicMax(scale_exp, (int)(mx >> 52));
    }
}

__global__ void split_kernel(const double *x, i64 ld, i64 r, i64 c, const int *scale_exp, float *hi, float *lo,
                             i64 ldo) {
    const int ef = *scale_exp;                         // biased exponent field of max |x|
    const double sc = (ef > 0) ? ldexp(1.0, 1023 - ef) : 1.0;   // brings max |x| into [1, 2)
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < r * c; e += (i64)gridDim.x * blockDim.x) {
        const i64 j = e / r, i = e - j * r;
        const double v = x[i + j * ld] * sc;           // exact (power of two)
        const float h = __double2float_rn(v);
        hi[i + j * ldo] = h;
        lo[i + j * ldo] = __double2float_rn(v - (double)h);
    }
}

// ------------------------------------------------------------------ the product kernel
// 64 x 64 output tile per 256-thread CTA, 4 x 4 outputs per thread (rows ty + 16 x, columns
// tx + 16 y), K staged 16 at a time; gridDim.z splits K (partial sums written as FP64 slabs and
// reduced by df64_reduce_kernel), else the epilogue applies alpha, beta and the scales.
constexpr int DB_M = 64, DB_N = 64, DB_K = 16;

// One multiply-add of the double-float product, on a pair of accumulators (rows x, x + 1 of one
// output column) with the packed FP32 instructions (FMUL2 / FFMA2 / FADD2): p = hi_a hi_b,
// e = fma(hi_a, hi_b, -p) exact; (s, c) += p by two-sum, c += e + hi_a lo_b + lo_a hi_b.
// renorm2: (s, c) <- two-sum(s, c) (no ordering assumption: a partial sum that cancels can
// leave |s| < |c|).
__device__ __forceinline__ float2 neg2(float2 v) { return make_float2(-v.x, -v.y); }
__device__ __forceinline__ void mac2(float2 ah, float2 al, float bh, float bl, float2 &s, float2 &c) {
    const float2 b = make_float2(bh, bh), bl2 = make_float2(bl, bl);
    const float2 p = __fmul2_rn(ah, b);
    const float2 e = __ffma2_rn(ah, b, neg2(p));
    const float2 t = __fadd2_rn(s, p);
    const float2 z = __fadd2_rn(t, neg2(s));
    const float2 err = __fadd2_rn(__fadd2_rn(s, neg2(__fadd2_rn(t, neg2(z)))), __fadd2_rn(p, neg2(z)));
    s = t;
    c = __fadd2_rn(c, __fadd2_rn(err, e));
    c = __ffma2_rn(ah, bl2, c);
    c = __ffma2_rn(al, b, c);
}
__device__ __forceinline__ void renorm2(float2 &s, float2 &c) {
    const float2 t = __fadd2_rn(s, c);
    const float2 z = __fadd2_rn(t, neg2(s));
    c = __fadd2_rn(__fadd2_rn(s, neg2(__fadd2_rn(t, neg2(z)))), __fadd2_rn(c, neg2(z)));
    s = t;
}

// One launch computes up to two products of the same shape and transposition (blockIdx.z = problem
// x K split); with `upper`, only the tiles on or above the diagonal (M == N, symmetric results).
struct Df64Prob {
    const float *Ah, *Al, *Bh, *Bl;
    i64 lda, ldb, ldc, ldo;
    const int *ea, *eb;
    double *C, *part;
    float *Oh, *Ol;
};
struct Df64Params {
    int M, N, K, kps, splits, nprob, upper;
    double alpha, beta;
    Df64Prob p[2];
};

template <bool TA, bool TB>
__global__ void __launch_bounds__(256) df64_gemm_kernel(const __grid_constant__ Df64Params P) {
    __shared__ float As[2][DB_K][DB_M + 1];
    __shared__ float Bs[2][DB_K][DB_N + 1];
    if (P.upper && blockIdx.x > blockIdx.y) return;
    const int prob = blockIdx.z / P.splits, split = blockIdx.z - prob * P.splits;
    const Df64Prob &Q = P.p[prob];
    const float *__restrict__ Ah = Q.Ah, *__restrict__ Al = Q.Al, *__restrict__ Bh = Q.Bh, *__restrict__ Bl = Q.Bl;
    const int M = P.M, N = P.N, K = P.K;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int m0 = blockIdx.x * DB_M, n0 = blockIdx.y * DB_N;
    const int kb = split * P.kps, ke = min(K, kb + P.kps);
    float s[4][4], c[4][4];
    float2 s2[2][4], c2[2][4];          // rows (2 xp, 2 xp + 1) of column y
#pragma unroll
    for (int x = 0; x < 2; x++)
#pragma unroll
        for (int y = 0; y < 4; y++) s2[x][y] = c2[x][y] = make_float2(0.f, 0.f);
    for (int k0 = kb; k0 < ke; k0 += DB_K) {
#pragma unroll
        for (int t = 0; t < (DB_M * DB_K) / 256; t++) {
            const int e = tid + 256 * t;
            int i, kk;
            if (!TA) { i = e % DB_M; kk = e / DB_M; }
            else { kk = e % DB_K; i = e / DB_K; }
            const int gi = m0 + i, gk = k0 + kk;
            float h = 0.f, l = 0.f;
            if (gi < M && gk < ke) {
                const i64 off = TA ? (gk + (i64)gi * Q.lda) : (gi + (i64)gk * Q.lda);
                h = Ah[off];
                l = Al[off];
            }
            As[0][kk][i] = h;
            As[1][kk][i] = l;
        }
#pragma unroll
        for (int t = 0; t < (DB_N * DB_K) / 256; t++) {
            const int e = tid + 256 * t;
            int j, kk;
            if (!TB) { kk = e % DB_K; j = e / DB_K; }
            else { j = e % DB_N; kk = e / DB_N; }
            const int gj = n0 + j, gk = k0 + kk;
            float h = 0.f, l = 0.f;
            if (gj < N && gk < ke) {
                const i64 off = TB ? (gj + (i64)gk * Q.ldb) : (gk + (i64)gj * Q.ldb);
                h = Bh[off];
                l = Bl[off];
            }
            Bs[0][kk][j] = h;
            Bs[1][kk][j] = l;
        }
        __syncthreads();
#pragma unroll 1
        for (int k4 = 0; k4 < DB_K; k4 += 4) {
#pragma unroll
            for (int kk = k4; kk < k4 + 4; kk++) {
                float ah[4], al[4], bh[4], bl[4];
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    ah[t] = As[0][kk][ty + 16 * t];
                    al[t] = As[1][kk][ty + 16 * t];
                    bh[t] = Bs[0][kk][tx + 16 * t];
                    bl[t] = Bs[1][kk][tx + 16 * t];
                }
#pragma unroll
                for (int x = 0; x < 2; x++) {
                    const float2 a2 = make_float2(ah[2 * x], ah[2 * x + 1]), l2 = make_float2(al[2 * x], al[2 * x + 1]);
#pragma unroll
                    for (int y = 0; y < 4; y++) mac2(a2, l2, bh[y], bl[y], s2[x][y], c2[x][y]);
                }
            }
#pragma unroll
            for (int x = 0; x < 2; x++)
#pragma unroll
                for (int y = 0; y < 4; y++) renorm2(s2[x][y], c2[x][y]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int x = 0; x < 2; x++)
#pragma unroll
        for (int y = 0; y < 4; y++) {
            s[2 * x][y] = s2[x][y].x; s[2 * x + 1][y] = s2[x][y].y;
            c[2 * x][y] = c2[x][y].x; c[2 * x + 1][y] = c2[x][y].y;
        }
    // undo the operand scales (exact powers of two)
    const int sa = *Q.ea, sb = *Q.eb;
    const double unscale = ldexp(1.0, (sa > 0 ? sa - 1023 : 0) + (sb > 0 ? sb - 1023 : 0));
#pragma unroll
    for (int x = 0; x < 4; x++) {
        const int gi = m0 + ty + 16 * x;
        if (gi >= M) continue;
#pragma unroll
        for (int y = 0; y < 4; y++) {
            const int gj = n0 + tx + 16 * y;
            if (gj >= N) continue;
            const double v = ((double)s[x][y] + (double)c[x][y]) * unscale;
            if (Q.part) {
                Q.part[(i64)split * M * N + gi + (i64)gj * M] = v;
            } else {
                double *cp = Q.C + gi + (i64)gj * Q.ldc;
                const double o = (P.beta == 0.0) ? P.alpha * v : P.alpha * v + P.beta * (*cp);
                *cp = o;
                if (Q.Oh) {
                    const float h = __double2float_rn(o);
                    Q.Oh[gi + (i64)gj * Q.ldo] = h;
                    Q.Ol[gi + (i64)gj * Q.ldo] = __double2float_rn(o - (double)h);
                }
            }
        }
    }
}

__global__ void df64_reduce_kernel(const __grid_constant__ Df64Params P) {
    const i64 MN = (i64)P.M * P.N;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < MN * P.nprob; e += (i64)gridDim.x * blockDim.x) {
        const int prob = (int)(e / MN);
        const i64 f = e - prob * MN;
        const i64 j = f / P.M, i = f - j * P.M;
        if (P.upper && (i / DB_M) > (j / DB_N)) continue;      // tile not computed
        const Df64Prob &Q = P.p[prob];
        double v = 0.0;
        for (int z = 0; z < P.splits; z++) v += Q.part[z * MN + f];
        double *cp = Q.C + i + j * Q.ldc;
        const double o = (P.beta == 0.0) ? P.alpha * v : P.alpha * v + P.beta * (*cp);
        *cp = o;
        if (Q.Oh) {
            const float h = __double2float_rn(o);
            Q.Oh[i + j * Q.ldo] = h;
            Q.Ol[i + j * Q.ldo] = __double2float_rn(o - (double)h);
        }
    }
}

unsigned grid_for(i64 n) {
    const i64 g = (n + 255) / 256;
    return (unsigned)std::max<i64>(1, std::min<i64>(g, (i64)std::max(1, ctx().sms) * 8));
}

}  // namespace

Df64Split::Df64Split(cudaStream_t s, DM<double> x, const int *exp_src) : r(x.r), c(x.c) {
    ld = pad_ld(r);
    buf = DBuf(sizeof(float) * (size_t)(2 * ld * std::max<i64>(c, 1)) + 16, s);
    hi = (float *)buf.get();
    lo = hi + ld * c;
    exp = (int *)(lo + ld * c);
    if (exp_src) {
        // a scale chosen by the caller (e.g. the scale of a factor of x): no max pass
        RSVD_CK(cudaMemcpyAsync(exp, exp_src, sizeof(int), cudaMemcpyDeviceToDevice, s));
    } else {
        RSVD_CK(cudaMemsetAsync(exp, 0, sizeof(int), s));
        if (r * c > 0) {
            maxexp_kernel<<<grid_for(r * c), 256, 0, s>>>(x.p, x.ld, r, c, exp);
            RSVD_LAUNCH_CK();
            ctx().launches++;
        }
    }
    if (r * c > 0) {
        split_kernel<<<grid_for(r * c), 256, 0, s>>>(x.p, x.ld, r, c, exp, hi, lo, ld);
        RSVD_LAUNCH_CK();
        ctx().launches++;
    }
}

// Up to two products of one shape: C_p = alpha op(A_p) op(B_p) + beta C_p.
static void df64_gemm_n(cudaStream_t s, bool ta, bool tb, double alpha, int nprob, const Df64View *A,
                        const Df64View *B, double beta, const DM<double> *C, const Df64Out *const *out, bool upper) {
    const i64 M = ta ? A[0].c : A[0].r, K = ta ? A[0].r : A[0].c;
    const i64 N = tb ? B[0].r : B[0].c;
    for (int q = 0; q < nprob; q++) {
        const i64 Mq = ta ? A[q].c : A[q].r, Kq = ta ? A[q].r : A[q].c;
        const i64 Nq = tb ? B[q].r : B[q].c, Kb = tb ? B[q].c : B[q].r;
        if (Mq != M || Kq != K || Nq != N || Kb != K || C[q].r != M || C[q].c != N)
            fail(RSVD_ERR_ARGUMENT, "df64_gemm: shape mismatch");
    }
    if (M == 0 || N == 0) return;
    if (M >= (1ll << 31) || N >= (1ll << 31) || K >= (1ll << 31)) fail(RSVD_ERR_ARGUMENT, "df64_gemm: too large");
    if (upper && M != N) fail(RSVD_ERR_ARGUMENT, "df64_gemm: upper needs a square result");
    const int mt = (int)ceil_div(M, DB_M), nt = (int)ceil_div(N, DB_N);
    if (nt > 65535) fail(RSVD_ERR_ARGUMENT, "df64_gemm: N too large for the tiling");
    const i64 tiles = upper ? (i64)mt * (mt + 1) / 2 : (i64)mt * nt;
    // split K until the grid covers the GPU (each split keeps >= 2 K steps of 16)
    const int sms = std::max(1, ctx().sms);
    int splits = 1;
    const int ksteps = (int)ceil_div(std::max<i64>(K, 1), DB_K);
    while (splits < 16 && tiles * nprob * splits < sms && ksteps / (2 * splits) >= 2) splits *= 2;
    const int kps = (int)(ceil_div(ksteps, splits) * DB_K);
    splits = (int)ceil_div(std::max<i64>(K, 1), kps);
    if ((i64)splits * nprob > 65535) fail(RSVD_ERR_ARGUMENT, "df64_gemm: grid too large");
    Df64Params P{};
    P.M = (int)M; P.N = (int)N; P.K = (int)K; P.kps = kps; P.splits = splits; P.nprob = nprob; P.upper = upper;
    P.alpha = alpha; P.beta = beta;
    DBuf pb;
    if (splits > 1) pb = DBuf(sizeof(double) * (size_t)(M * N * splits * nprob), s);
    for (int q = 0; q < nprob; q++) {
        Df64Prob &Q = P.p[q];
        Q.Ah = A[q].hi; Q.Al = A[q].lo; Q.lda = A[q].ld; Q.ea = A[q].exp;
        Q.Bh = B[q].hi; Q.Bl = B[q].lo; Q.ldb = B[q].ld; Q.eb = B[q].exp;
        Q.C = C[q].p; Q.ldc = C[q].ld;
        Q.part = splits > 1 ? (double *)pb.get() + (size_t)q * M * N * splits : nullptr;
        Q.Oh = out && out[q] ? out[q]->hi : nullptr;
        Q.Ol = out && out[q] ? out[q]->lo : nullptr;
        Q.ldo = out && out[q] ? out[q]->ld : 0;
    }
    dim3 grid(mt, nt, splits * nprob);
    if (!ta && !tb) df64_gemm_kernel<false, false><<<grid, 256, 0, s>>>(P);
    else if (ta && !tb) df64_gemm_kernel<true, false><<<grid, 256, 0, s>>>(P);
    else if (!ta && tb) df64_gemm_kernel<false, true><<<grid, 256, 0, s>>>(P);
    else df64_gemm_kernel<true, true><<<grid, 256, 0, s>>>(P);
    RSVD_LAUNCH_CK();
    ctx().launches++;
    if (splits > 1) {
        df64_reduce_kernel<<<grid_for(M * N * nprob), 256, 0, s>>>(P);
        RSVD_LAUNCH_CK();
        ctx().launches++;
    }
}

void df64_gemm(cudaStream_t s, bool ta, bool tb, double alpha, Df64View A, Df64View B, double beta, DM<double> C,
               const Df64Out *out) {
    const Df64Out *o[1] = {out};
    df64_gemm_n(s, ta, tb, alpha, 1, &A, &B, beta, &C, o, false);
}

void df64_gram_pair(cudaStream_t s, Df64View A0, DM<double> C0, Df64View A1, DM<double> C1) {
    const Df64View A[2] = {A0, A1};
    const DM<double> C[2] = {C0, C1};
    df64_gemm_n(s, true, false, 1.0, 2, A, A, 0.0, C, nullptr, true);
}

void df64_gemm(cudaStream_t s, bool ta, bool tb, double alpha, const Df64Split &A, const Df64Split &B, double beta,
               DM<double> C) {
    df64_gemm(s, ta, tb, alpha, A.view(), B.view(), beta, C, nullptr);
}

}  // namespace rsvd
