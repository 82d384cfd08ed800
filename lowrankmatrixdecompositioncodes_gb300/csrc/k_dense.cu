// k_dense.cu -- CUDA-core kernels of the engine: SIMT GEMM (FP64 / FP32), layout
// helpers, Philox Gaussian test matrices, norms, Gram, Cholesky, triangular solves,
// one-sided Jacobi SVD and a Householder QR fallback.
//
// These carry the FP64 path that reproduces the reference (every product the
// reference does with cblas_dgemm, multi_core_mkl_code/matrix_vector_functions_intel_mkl.c:538-561)
// and the small k x k FP64 work of every precision mode.
#include "rsvd_internal.h"
#include "k_common.cuh"

#include <algorithm>
#include <cstdint>
#include <type_traits>
#include <cmath>

namespace rsvd {

// =====================================================================================
// SIMT GEMM:  C = alpha * op(A) * op(B) + beta * C, column-major.
// 64x64 output tile per 256-thread block, 4x4 per thread, K staged 16 at a time.
// =====================================================================================
namespace {
constexpr int GB_M = 64, GB_N = 64, GB_K = 16;

template <typename T, bool TA, bool TB>
__global__ void __launch_bounds__(256) gemm_simt_kernel(i64 M, i64 N, i64 K, T alpha,
                                                        const T *__restrict__ A, i64 lda,
                                                        const T *__restrict__ B, i64 ldb, T beta,
                                                        T *__restrict__ C, i64 ldc) {
    __shared__ T As[GB_K][GB_M + 1];
    __shared__ T Bs[GB_K][GB_N + 1];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const i64 m0 = (i64)blockIdx.x * GB_M, n0 = (i64)blockIdx.y * GB_N;
    T acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = T(0);

    for (i64 k0 = 0; k0 < K; k0 += GB_K) {
#pragma unroll
        for (int e = tid; e < GB_M * GB_K; e += 256) {
            int i, kk;
            if (!TA) { i = e % GB_M; kk = e / GB_M; }
            else { kk = e % GB_K; i = e / GB_K; }
            const i64 gi = m0 + i, gk = k0 + kk;
            T v = T(0);
            if (gi < M && gk < K) v = TA ? A[gk + gi * lda] : A[gi + gk * lda];
            As[kk][i] = v;
        }
#pragma unroll
        for (int e = tid; e < GB_N * GB_K; e += 256) {
            int j, kk;
            if (!TB) { kk = e % GB_K; j = e / GB_K; }
            else { j = e % GB_N; kk = e / GB_N; }
            const i64 gj = n0 + j, gk = k0 + kk;
            T v = T(0);
            if (gj < N && gk < K) v = TB ? B[gj + gk * ldb] : B[gk + gj * ldb];
            Bs[kk][j] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GB_K; kk++) {
            T a[4], b[4];
#pragma unroll
            for (int t = 0; t < 4; t++) a[t] = As[kk][ty + 16 * t];
#pragma unroll
            for (int t = 0; t < 4; t++) b[t] = Bs[kk][tx + 16 * t];
#pragma unroll
            for (int x = 0; x < 4; x++)
#pragma unroll
                for (int y = 0; y < 4; y++) acc[x][y] = fma(a[x], b[y], acc[x][y]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int x = 0; x < 4; x++) {
        const i64 gi = m0 + ty + 16 * x;
        if (gi >= M) continue;
#pragma unroll
        for (int y = 0; y < 4; y++) {
            const i64 gj = n0 + tx + 16 * y;
            if (gj >= N) continue;
            T *c = C + gi + gj * ldc;
            *c = (beta == T(0)) ? alpha * acc[x][y] : alpha * acc[x][y] + beta * (*c);
        }
    }
}
}  // namespace

// FP32 CUDA-core GEMM for op(B) = B: 128 x 64 tile, 256 threads, 8 x 4 outputs per thread
// (rows ty*4+{0..3} and 64+ty*4+{0..3}, columns tx*4+{0..3}), K staged 16 at a time with
// the next stage prefetched into registers while the current one is consumed.
template <bool TA>
__global__ void __launch_bounds__(256) sgemm_128x64_kernel(i64 M, i64 N, i64 K, float alpha,
                                                           const float *__restrict__ A, i64 lda,
                                                           const float *__restrict__ B, i64 ldb, float beta,
                                                           float *__restrict__ C, i64 ldc) {
    __shared__ __align__(16) float As[16][128];
    __shared__ __align__(16) float Bs[16][64];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const i64 m0 = (i64)blockIdx.x * 128, n0 = (i64)blockIdx.y * 64;
    float ra[8], rb[4];
    auto load = [&](i64 k0) {
#pragma unroll
        for (int e = 0; e < 8; e++) {
            const int idx = tid + 256 * e;
            int i, kk;
            if (!TA) { i = idx & 127; kk = idx >> 7; }
            else { kk = idx & 15; i = idx >> 4; }
            const i64 gi = m0 + i, gk = k0 + kk;
            ra[e] = (gi < M && gk < K) ? (TA ? A[gk + gi * lda] : A[gi + gk * lda]) : 0.f;
        }
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int idx = tid + 256 * e;
            const int kk = idx & 15, j = idx >> 4;
            const i64 gj = n0 + j, gk = k0 + kk;
            rb[e] = (gj < N && gk < K) ? B[gk + gj * ldb] : 0.f;
        }
    };
    auto store = [&]() {
#pragma unroll
        for (int e = 0; e < 8; e++) {
            const int idx = tid + 256 * e;
            int i, kk;
            if (!TA) { i = idx & 127; kk = idx >> 7; }
            else { kk = idx & 15; i = idx >> 4; }
            As[kk][i] = ra[e];
        }
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int idx = tid + 256 * e;
            Bs[idx & 15][idx >> 4] = rb[e];
        }
    };
    // accumulators as row pairs (rows x, x+1 of column y) for packed FP32 FMAs (FFMA2):
    // the A operand pairs come straight from the float4 loads, only B is broadcast
    float2 acc2[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc2[a][b] = make_float2(0.f, 0.f);
    load(0);
    for (i64 k0 = 0; k0 < K; k0 += 16) {
        store();
        __syncthreads();
        if (k0 + 16 < K) load(k0 + 16);
#pragma unroll
        for (int kk = 0; kk < 16; kk++) {
            const float4 a0 = *reinterpret_cast<const float4 *>(&As[kk][ty * 4]);
            const float4 a1 = *reinterpret_cast<const float4 *>(&As[kk][64 + ty * 4]);
            const float4 b0 = *reinterpret_cast<const float4 *>(&Bs[kk][tx * 4]);
            const float2 ap[4] = {make_float2(a0.x, a0.y), make_float2(a0.z, a0.w), make_float2(a1.x, a1.y),
                                  make_float2(a1.z, a1.w)};
            const float2 bp[4] = {make_float2(b0.x, b0.x), make_float2(b0.y, b0.y), make_float2(b0.z, b0.z),
                                  make_float2(b0.w, b0.w)};
#pragma unroll
            for (int x = 0; x < 4; x++)
#pragma unroll
                for (int y = 0; y < 4; y++) acc2[x][y] = __ffma2_rn(ap[x], bp[y], acc2[x][y]);
        }
        __syncthreads();
    }
    float acc[8][4];
#pragma unroll
    for (int x = 0; x < 4; x++)
#pragma unroll
        for (int y = 0; y < 4; y++) {
            acc[2 * x][y] = acc2[x][y].x;
            acc[2 * x + 1][y] = acc2[x][y].y;
        }
#pragma unroll
    for (int x = 0; x < 8; x++) {
        const i64 gi = m0 + (x < 4 ? ty * 4 + x : 64 + ty * 4 + (x - 4));
        if (gi >= M) continue;
#pragma unroll
        for (int y = 0; y < 4; y++) {
            const i64 gj = n0 + tx * 4 + y;
            if (gj >= N) continue;
            float *c = C + gi + gj * ldc;
            *c = (beta == 0.f) ? alpha * acc[x][y] : alpha * acc[x][y] + beta * (*c);
        }
    }
}

template <typename T>
void gemm_simt(cudaStream_t s, bool ta, bool tb, i64 M, i64 N, i64 K, T alpha, const T *A,
               i64 lda, const T *B, i64 ldb, T beta, T *C, i64 ldc) {
    if (M <= 0 || N <= 0) return;
    if (std::is_same<T, float>::value && !tb && M >= 128) {
        dim3 grid(ceil_div(M, 128), ceil_div(N, 64));
        if (grid.y <= 65535) {
            if (ta) sgemm_128x64_kernel<true><<<grid, 256, 0, s>>>(M, N, K, (float)alpha, (const float *)A, lda,
                                                                  (const float *)B, ldb, (float)beta, (float *)C, ldc);
            else sgemm_128x64_kernel<false><<<grid, 256, 0, s>>>(M, N, K, (float)alpha, (const float *)A, lda,
                                                                (const float *)B, ldb, (float)beta, (float *)C, ldc);
            RSVD_LAUNCH_CK();
            ctx().launches++;
            return;
        }
    }
    dim3 grid(ceil_div(M, GB_M), ceil_div(N, GB_N));
    if (grid.y > 65535) fail(RSVD_ERR_ARGUMENT, "gemm: N too large for the SIMT tiling");
    if (!ta && !tb) gemm_simt_kernel<T, false, false><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
    else if (ta && !tb) gemm_simt_kernel<T, true, false><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
    else if (!ta && tb) gemm_simt_kernel<T, false, true><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
    else gemm_simt_kernel<T, true, true><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
    RSVD_LAUNCH_CK();
    ctx().launches++;
}

template <typename T>
void gemm(cudaStream_t s, bool ta, bool tb, T alpha, DM<T> A, DM<T> B, T beta, DM<T> C) {
    const i64 M = ta ? A.c : A.r, K = ta ? A.r : A.c;
    const i64 N = tb ? B.r : B.c, Kb = tb ? B.c : B.r;
    if (K != Kb || C.r != M || C.c != N) fail(RSVD_ERR_ARGUMENT, "gemm: shape mismatch");
    gemm_simt<T>(s, ta, tb, M, N, K, alpha, A.p, A.ld, B.p, B.ld, beta, C.p, C.ld);
}

template void gemm_simt<double>(cudaStream_t, bool, bool, i64, i64, i64, double, const double *, i64,
                                const double *, i64, double, double *, i64);
template void gemm_simt<float>(cudaStream_t, bool, bool, i64, i64, i64, float, const float *, i64,
                               const float *, i64, float, float *, i64);
template void gemm<double>(cudaStream_t, bool, bool, double, DM<double>, DM<double>, double, DM<double>);
template void gemm<float>(cudaStream_t, bool, bool, float, DM<float>, DM<float>, float, DM<float>);

// =====================================================================================
// Layout helpers
// =====================================================================================
namespace {
template <typename Ts, typename Td>
// 2-D launch: blockIdx.x covers 1024 rows (4 per thread, coalesced), blockIdx.y strides columns
__global__ void convert_kernel(const Ts *src, i64 lds, Td *dst, i64 ldd, i64 r, i64 c) {
    const i64 i0 = (i64)blockIdx.x * 1024 + threadIdx.x;
    for (i64 j = blockIdx.y; j < c; j += gridDim.y) {
        const Ts *sc = src + j * lds;
        Td *dc = dst + j * ldd;
        Ts v[4];
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const i64 i = i0 + 256 * t;
            v[t] = (i < r) ? sc[i] : Ts(0);
        }
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const i64 i = i0 + 256 * t;
            if (i < r) dc[i] = (Td)v[t];
        }
    }
}
// Contiguous FP32 -> BF16 (the per-call BF16 copy of a dense operand): 16-byte loads, four per
// thread in flight, 8-byte stores, a grid-stride loop over ~8 CTAs per SM; the n % 4 tail by
// the first threads.  Round to nearest even, as convert_kernel.
__global__ void convert_f32_bf16_flat_kernel(const float *__restrict__ src, __nv_bfloat16 *__restrict__ dst, i64 n) {
    const i64 n4 = n >> 2, stride = (i64)gridDim.x * blockDim.x;
    const float4 *s4 = reinterpret_cast<const float4 *>(src);
    uint2 *d4 = reinterpret_cast<uint2 *>(dst);
    auto pack = [](float4 v) {
        const __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y), b = __floats2bfloat162_rn(v.z, v.w);
        return make_uint2(*reinterpret_cast<const uint32_t *>(&a), *reinterpret_cast<const uint32_t *>(&b));
    };
    i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n4; i += 4 * stride) {
        float4 v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) v[u] = __ldcs(s4 + i + u * stride);
#pragma unroll
        for (int u = 0; u < 4; u++) d4[i + u * stride] = pack(v[u]);
    }
    for (; i < n4; i += stride) d4[i] = pack(__ldcs(s4 + i));
    const i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n - 4 * n4) dst[4 * n4 + t] = __float2bfloat16_rn(src[4 * n4 + t]);
}
// dst = (float)src and dst2 = bf16(dst) in one pass (the C-API upload of a matrix whose BF16
// copy the tensor-core products will read: the second output rides on the link-bound read).
template <typename Ts>
__global__ void convert_f32_bf16_kernel(const Ts *src, i64 lds, float *dst, i64 ldd, __nv_bfloat16 *dst2, i64 ldd2,
                                        i64 r, i64 c) {
    const i64 i0 = (i64)blockIdx.x * 1024 + threadIdx.x;
    for (i64 j = blockIdx.y; j < c; j += gridDim.y) {
        const Ts *sc = src + j * lds;
        Ts v[4];
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const i64 i = i0 + 256 * t;
            v[t] = (i < r) ? sc[i] : Ts(0);
        }
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const i64 i = i0 + 256 * t;
            if (i < r) {
                const float f = (float)v[t];
                dst[i + j * ldd] = f;
                dst2[i + j * ldd2] = __float2bfloat16_rn(f);
            }
        }
    }
}
template <typename T>
__global__ void fill_kernel(T *a, i64 ld, i64 r, i64 c, int identity) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < r * c; e += (i64)gridDim.x * blockDim.x) {
        const i64 i = e % r, j = e / r;
        a[i + j * ld] = (identity && i == j) ? T(1) : T(0);
    }
}
template <typename T>
__global__ void transpose_kernel(const T *src, i64 lds, T *dst, i64 ldd, i64 r, i64 c) {
    __shared__ T tile[32][33];
    const i64 i0 = (i64)blockIdx.x * 32, j0 = (i64)blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += 8) {
        const i64 i = i0 + threadIdx.x, j = j0 + y;
        if (i < r && j < c) tile[y][threadIdx.x] = src[i + j * lds];
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += 8) {
        const i64 j = j0 + threadIdx.x, i = i0 + y;   // dst(j, i) = src(i, j)
        if (i < r && j < c) dst[j + i * ldd] = tile[threadIdx.x][y];
    }
}
template <typename T>
__global__ void gather_cols_kernel(const T *src, i64 lds, const int *idx, T *dst, i64 ldd, i64 r, i64 c) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < r * c; e += (i64)gridDim.x * blockDim.x) {
        const i64 i = e % r, j = e / r;
        dst[i + j * ldd] = src[i + (i64)idx[j] * lds];
    }
}
template <typename T>
__global__ void gather_rows_kernel(const T *src, i64 lds, const int *idx, T *dst, i64 ldd, i64 r, i64 c) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < r * c; e += (i64)gridDim.x * blockDim.x) {
        const i64 i = e % r, j = e / r;
        dst[i + j * ldd] = src[(i64)idx[i] + j * lds];
    }
}
template <typename T>
__global__ void sub_kernel(T *a, i64 lda, const T *b, i64 ldb, i64 r, i64 c) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < r * c; e += (i64)gridDim.x * blockDim.x) {
        const i64 i = e % r, j = e / r;
        a[i + j * lda] -= b[i + j * ldb];
    }
}
template <typename T>
// Sum of squares, 2-D like convert_kernel (blockIdx.x: 1024 rows, blockIdx.y strides the
// columns).  Each thread sums its elements in T with Kahan compensation and converts once:
// FP32 data costs no FP64 arithmetic per element (GB300's FP64 rate is a small fraction of
// its FP32 rate), and the compensated FP32 sum keeps ~2^-24 relative accuracy.
__global__ void sumsq_kernel(const T *a, i64 ld, i64 r, i64 c, double *partial) {
    __shared__ double sc[32];
    const i64 i0 = (i64)blockIdx.x * 1024 + threadIdx.x;
    T sum = T(0), comp = T(0);
    for (i64 j = blockIdx.y; j < c; j += gridDim.y) {
        const T *col = a + j * ld;
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const i64 i = i0 + 256 * t;
            if (i < r) {
                const T v = col[i];
                const T y = v * v - comp;
                const T tt = sum + y;
                comp = (tt - sum) - y;
                sum = tt;
            }
        }
    }
    double acc = block_sum((double)sum - (double)comp, sc);
    if (threadIdx.x == 0) partial[blockIdx.x + (i64)gridDim.x * blockIdx.y] = acc;
}
unsigned grid_for(i64 n) {
    i64 g = (n + 255) / 256;
    const i64 cap = (i64)std::max(1, ctx().sms) * 16;
    return (unsigned)std::max<i64>(1, std::min(g, cap));
}
}  // namespace

namespace {
// Same 2-D layout as convert_kernel: hi = bf16(x), lo = bf16(x - hi).
__global__ void split_bf16_kernel(const float *src, i64 lds, __nv_bfloat16 *hi, i64 ldh, __nv_bfloat16 *lo, i64 ldl,
                                  i64 r, i64 c) {
    const i64 i0 = (i64)blockIdx.x * 1024 + threadIdx.x;
    for (i64 j = blockIdx.y; j < c; j += gridDim.y) {
        float v[4];
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const i64 i = i0 + 256 * t;
            v[t] = (i < r) ? src[i + j * lds] : 0.f;
        }
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const i64 i = i0 + 256 * t;
            if (i < r) {
                const __nv_bfloat16 h = __float2bfloat16_rn(v[t]);
                hi[i + j * ldh] = h;
                lo[i + j * ldl] = __float2bfloat16_rn(v[t] - __bfloat162float(h));
            }
        }
    }
}
}  // namespace

void split_bf16(cudaStream_t s, DM<float> src, DM<__nv_bfloat16> hi, DM<__nv_bfloat16> lo) {
    if (src.r * src.c == 0) return;
    const dim3 grid((unsigned)((src.r + 1023) / 1024), (unsigned)std::min<i64>(src.c, 65535));
    split_bf16_kernel<<<grid, 256, 0, s>>>(src.p, src.ld, hi.p, hi.ld, lo.p, lo.ld, src.r, src.c);
    RSVD_LAUNCH_CK();
    ctx().launches++;
}

template <typename Ts, typename Td>
void convert(cudaStream_t s, DM<Ts> src, DM<Td> dst) {
    if (src.r * src.c == 0) return;
    if constexpr (std::is_same<Ts, float>::value && std::is_same<Td, __nv_bfloat16>::value) {
        if ((src.ld == src.r || src.c == 1) && (dst.ld == dst.r || dst.c == 1) &&
            reinterpret_cast<uintptr_t>(src.p) % 16 == 0 && reinterpret_cast<uintptr_t>(dst.p) % 8 == 0) {
            const i64 n = src.r * src.c;
            const i64 blocks = std::max<i64>(1, std::min<i64>((n / 4 + 255) / 256, (i64)std::max(1, ctx().sms) * 8));
            convert_f32_bf16_flat_kernel<<<(unsigned)blocks, 256, 0, s>>>(src.p, dst.p, n);
            RSVD_LAUNCH_CK();
            ctx().launches++;
            return;
        }
    }
    const dim3 grid((unsigned)((src.r + 1023) / 1024), (unsigned)std::min<i64>(src.c, 65535));
    convert_kernel<Ts, Td><<<grid, 256, 0, s>>>(src.p, src.ld, dst.p, dst.ld, src.r, src.c);
    RSVD_LAUNCH_CK();
    ctx().launches++;
}
template <typename Ts>
void convert_f32_bf16(cudaStream_t s, DM<Ts> src, DM<float> dst, DM<__nv_bfloat16> dst2) {
    if (src.r * src.c == 0) return;
    const dim3 grid((unsigned)((src.r + 1023) / 1024), (unsigned)std::min<i64>(src.c, 65535));
    convert_f32_bf16_kernel<Ts><<<grid, 256, 0, s>>>(src.p, src.ld, dst.p, dst.ld, dst2.p, dst2.ld, src.r, src.c);
    RSVD_LAUNCH_CK();
    ctx().launches++;
}
template void convert_f32_bf16<double>(cudaStream_t, DM<double>, DM<float>, DM<__nv_bfloat16>);
template void convert_f32_bf16<float>(cudaStream_t, DM<float>, DM<float>, DM<__nv_bfloat16>);
template void convert<double, float>(cudaStream_t, DM<double>, DM<float>);
template void convert<float, double>(cudaStream_t, DM<float>, DM<double>);
template void convert<double, double>(cudaStream_t, DM<double>, DM<double>);
template void convert<float, float>(cudaStream_t, DM<float>, DM<float>);
template void convert<float, __nv_bfloat16>(cudaStream_t, DM<float>, DM<__nv_bfloat16>);
template void convert<double, __nv_bfloat16>(cudaStream_t, DM<double>, DM<__nv_bfloat16>);

template <typename T>
void fill_zero(cudaStream_t s, DM<T> a) {
    if (a.r * a.c == 0) return;
    fill_kernel<T><<<grid_for(a.r * a.c), 256, 0, s>>>(a.p, a.ld, a.r, a.c, 0);
    RSVD_LAUNCH_CK();
}
template <typename T>
void set_identity(cudaStream_t s, DM<T> a) {
    if (a.r * a.c == 0) return;
    fill_kernel<T><<<grid_for(a.r * a.c), 256, 0, s>>>(a.p, a.ld, a.r, a.c, 1);
    RSVD_LAUNCH_CK();
}
template <typename T>
void transpose(cudaStream_t s, DM<T> src, DM<T> dst) {
    if (dst.r != src.c || dst.c != src.r) fail(RSVD_ERR_ARGUMENT, "transpose: shape mismatch");
    if (src.r * src.c == 0) return;
    dim3 grid(ceil_div(src.r, 32), ceil_div(src.c, 32));
    transpose_kernel<T><<<grid, dim3(32, 8), 0, s>>>(src.p, src.ld, dst.p, dst.ld, src.r, src.c);
    RSVD_LAUNCH_CK();
}
template <typename T>
void gather_cols(cudaStream_t s, DM<T> src, const int *idx, DM<T> dst) {
    if (dst.r * dst.c == 0) return;
    gather_cols_kernel<T><<<grid_for(dst.r * dst.c), 256, 0, s>>>(src.p, src.ld, idx, dst.p, dst.ld, dst.r, dst.c);
    RSVD_LAUNCH_CK();
}
template <typename T>
void gather_rows(cudaStream_t s, DM<T> src, const int *idx, DM<T> dst) {
    if (dst.r * dst.c == 0) return;
    gather_rows_kernel<T><<<grid_for(dst.r * dst.c), 256, 0, s>>>(src.p, src.ld, idx, dst.p, dst.ld, dst.r, dst.c);
    RSVD_LAUNCH_CK();
}
template <typename T>
void sub_inplace(cudaStream_t s, DM<T> a, DM<T> b) {
    if (a.r * a.c == 0) return;
    sub_kernel<T><<<grid_for(a.r * a.c), 256, 0, s>>>(a.p, a.ld, b.p, b.ld, a.r, a.c);
    RSVD_LAUNCH_CK();
}
template <typename T>
double frob_norm(cudaStream_t s, DM<T> a) {
    if (a.r * a.c == 0) return 0.0;
    const unsigned gx = (unsigned)((a.r + 1023) / 1024);
    const unsigned gy = (unsigned)std::max<i64>(1, std::min<i64>(a.c, std::max<i64>(1, (i64)std::max(1, ctx().sms) * 8 / gx)));
    const unsigned g = gx * gy;
    DBuf part(sizeof(double) * g, s);
    sumsq_kernel<T><<<dim3(gx, gy), 256, 0, s>>>(a.p, a.ld, a.r, a.c, (double *)part.get());
    RSVD_LAUNCH_CK();
    std::vector<double> h(g);
    RSVD_CK(cudaMemcpyAsync(h.data(), part.get(), sizeof(double) * g, cudaMemcpyDeviceToHost, s));
    RSVD_CK(cudaStreamSynchronize(s));
    double acc = 0.0;
    for (double v : h) acc += v;
    return std::sqrt(acc);
}

#define RSVD_INST_LAYOUT(T)                                              \
    template void fill_zero<T>(cudaStream_t, DM<T>);                     \
    template void set_identity<T>(cudaStream_t, DM<T>);                  \
    template void transpose<T>(cudaStream_t, DM<T>, DM<T>);              \
    template void gather_cols<T>(cudaStream_t, DM<T>, const int *, DM<T>); \
    template void gather_rows<T>(cudaStream_t, DM<T>, const int *, DM<T>); \
    template void sub_inplace<T>(cudaStream_t, DM<T>, DM<T>);            \
    template double frob_norm<T>(cudaStream_t, DM<T>);
RSVD_INST_LAYOUT(double)
RSVD_INST_LAYOUT(float)

// =====================================================================================
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) + Box-Muller Gaussians.
// Element e of the column-major matrix uses counter (e/4, offset) and key seed; the
// values are rounded through float, like the reference's float Gaussians.
// =====================================================================================
namespace {
struct U4 { uint32_t x, y, z, w; };
__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}
template <typename T>
__global__ void philox_kernel(uint64_t seed, uint64_t offset, T *out, i64 ld, i64 r, i64 c) {
    const i64 n = r * c, groups = (n + 3) / 4;
    for (i64 g = blockIdx.x * (i64)blockDim.x + threadIdx.x; g < groups; g += (i64)gridDim.x * blockDim.x) {
        const U4 v = philox4x32_10(U4{(uint32_t)g, (uint32_t)(g >> 32), (uint32_t)offset, (uint32_t)(offset >> 32)},
                                   (uint32_t)seed, (uint32_t)(seed >> 32));
        const uint32_t u[4] = {v.x, v.y, v.z, v.w};
        // Box-Muller in FP32 (the values are FP32 in every mode; FP64 transcendental
        // throughput is low on this part).  Same formulas as the batched kernel's generator.
        float z[4];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const float u1 = ((float)u[2 * h] + 1.0f) * 2.3283064365386963e-10f;   // (0,1]
            const float u2 = (float)u[2 * h + 1] * 2.3283064365386963e-10f;       // [0,1)
            const float rad = sqrtf(-2.0f * logf(u1));
            float sn, cs;
            sincospif(2.0f * u2, &sn, &cs);
            z[2 * h] = rad * cs;
            z[2 * h + 1] = rad * sn;
        }
        const i64 e0 = 4 * g;
        i64 col = e0 / r, row = e0 - col * r;
#pragma unroll
        for (int t = 0; t < 4; t++) {
            if (e0 + t < n) {
                out[row + col * ld] = (T)z[t];
                if (++row == r) { row = 0; ++col; }
            }
        }
    }
}
}  // namespace

void philox_gaussian(cudaStream_t s, unsigned long long seed, unsigned long long offset, DM<double> out) {
    if (out.r * out.c == 0) return;
    philox_kernel<double><<<grid_for((out.r * out.c + 3) / 4), 256, 0, s>>>(seed, offset, out.p, out.ld, out.r, out.c);
    RSVD_LAUNCH_CK();
}
void philox_gaussian(cudaStream_t s, unsigned long long seed, unsigned long long offset, DM<float> out) {
    if (out.r * out.c == 0) return;
    philox_kernel<float><<<grid_for((out.r * out.c + 3) / 4), 256, 0, s>>>(seed, offset, out.p, out.ld, out.r, out.c);
    RSVD_LAUNCH_CK();
}

// =====================================================================================
// Cholesky G = R^T R (upper), FP64, one 1024-thread block, right-looking by column.
// =====================================================================================
namespace {
// A pivot d_j is a breakdown when d_j <= rel_tol * G_jj(original): column j is then
// numerically inside the span of the earlier columns at the Gram's precision.
__global__ void __launch_bounds__(1024) cholesky_kernel(double *G, i64 ld, int n, double rel_tol, int *flag) {
    extern __shared__ double diag0[];
    __shared__ double piv;
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) diag0[j] = G[j + j * ld];
    __syncthreads();
    for (int j = 0; j < n; j++) {
        if (threadIdx.x == 0) {
            const double d = G[j + j * ld];
            if (!isfinite(d) || !(d > 0.0) || !(d > rel_tol * diag0[j])) { bad = 1; piv = 1.0; }
            else piv = sqrt(d);
            G[j + j * ld] = piv;
        }
        __syncthreads();
        if (bad) break;
        const double p = piv;
        for (int k = j + 1 + threadIdx.x; k < n; k += blockDim.x) G[j + k * ld] /= p;
        __syncthreads();
        // trailing upper update: G(i,k) -= R(j,i) R(j,k) for j < i <= k
        const int t = n - j - 1;
        const i64 cnt = (i64)t * (t + 1) / 2;
        for (i64 e = threadIdx.x; e < cnt; e += blockDim.x) {
            // map e -> (i,k) with i <= k over the t x t upper triangle, column-major packing
            int kk = (int)((sqrt(8.0 * (double)e + 1.0) - 1.0) * 0.5);
            while ((i64)kk * (kk + 1) / 2 > e) kk--;
            while ((i64)(kk + 1) * (kk + 2) / 2 <= e) kk++;
            const int ii = (int)(e - (i64)kk * (kk + 1) / 2);
            const int i = j + 1 + ii, k = j + 1 + kk;
            G[i + k * ld] -= G[j + i * ld] * G[j + k * ld];
        }
        __syncthreads();
    }
    __syncthreads();
    if (bad) {
        if (threadIdx.x == 0) atomicExch(flag, 1);
        return;
    }
    for (i64 e = threadIdx.x; e < (i64)n * n; e += blockDim.x) {
        const int i = (int)(e % n), k = (int)(e / n);
        if (i > k) G[i + k * ld] = 0.0;
    }
}
}  // namespace

bool cholesky_upper(cudaStream_t s, DM<double> G, double rel_tol, int *d_flag) {
    if (G.r != G.c) fail(RSVD_ERR_ARGUMENT, "cholesky: not square");
    if (G.r > 6000) fail(RSVD_ERR_ARGUMENT, "cholesky: order above 6000");
    RSVD_CK(cudaMemsetAsync(d_flag, 0, sizeof(int), s));
    const size_t shm = sizeof(double) * (size_t)G.r;
    if (shm > 48 * 1024) RSVD_CK(cudaFuncSetAttribute(cholesky_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
    cholesky_kernel<<<1, 1024, shm, s>>>(G.p, G.ld, (int)G.r, rel_tol, d_flag);
    RSVD_LAUNCH_CK();
    int h = 0;
    RSVD_CK(cudaMemcpyAsync(&h, d_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    RSVD_CK(cudaStreamSynchronize(s));
    return h == 0;
}

// =====================================================================================
// Triangular solves
// =====================================================================================
namespace {
// Q(i,:) = Y(i,:) * R^{-1}, one thread per row; Q may alias Y.
template <typename T>
__global__ void trsm_right_upper_kernel(const T *Y, i64 ldy, const double *R, i64 ldr, T *Q, i64 ldq,
                                        i64 m, int c) {
    const i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x;
    if (i >= m) return;
    for (int j = 0; j < c; j++) {
        double acc = (double)Y[i + j * ldy];
        for (int t = 0; t < j; t++) acc -= (double)Q[i + t * ldq] * R[t + j * ldr];
        Q[i + j * ldq] = (T)(acc / R[j + j * ldr]);
    }
}
// X(:,b) = R^{-1} B(:,b), one warp per column (back substitution, lane-parallel dot).
__global__ void trsm_left_upper_kernel(const double *R, i64 ldr, const double *B, i64 ldb, double *X,
                                       i64 ldx, int k, i64 ncols) {
    const i64 col = (blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (col >= ncols) return;
    double *x = X + col * ldx;
    const double *b = B + col * ldb;
    if (x != b)
        for (int i = lane; i < k; i += 32) x[i] = b[i];
    __syncwarp();
    for (int j = k - 1; j >= 0; j--) {
        double xj = 0.0;
        if (lane == 0) xj = x[j] / R[j + j * ldr];
        xj = __shfl_sync(0xffffffffu, xj, 0);
        for (int i = lane; i < j; i += 32) x[i] -= R[i + j * ldr] * xj;
        if (lane == 0) x[j] = xj;
        __syncwarp();
    }
}
}  // namespace

template <typename T>
void trsm_right_upper(cudaStream_t s, DM<T> Y, DM<double> R, DM<T> Q) {
    if (Y.r == 0) return;
    trsm_right_upper_kernel<T><<<ceil_div(Y.r, 128), 128, 0, s>>>(Y.p, Y.ld, R.p, R.ld, Q.p, Q.ld, Y.r, (int)Y.c);
    RSVD_LAUNCH_CK();
}
template void trsm_right_upper<double>(cudaStream_t, DM<double>, DM<double>, DM<double>);
template void trsm_right_upper<float>(cudaStream_t, DM<float>, DM<double>, DM<float>);

void trsm_left_upper(cudaStream_t s, DM<double> R, DM<double> B, DM<double> X) {
    if (B.c == 0 || B.r == 0) return;
    const i64 threads = B.c * 32;
    trsm_left_upper_kernel<<<ceil_div(threads, 256), 256, 0, s>>>(R.p, R.ld, B.p, B.ld, X.p, X.ld, (int)B.r, B.c);
    RSVD_LAUNCH_CK();
}

// =====================================================================================
// One-sided (Hestenes) Jacobi SVD of an n x n FP64 matrix, one 1024-thread block.
// Columns of W = G V are orthogonalised by plane rotations in round-robin order
// until no pair has |w_p.w_q| > tol * |w_p| |w_q|.  Then sv_j = |w_j|, U = W / sv,
// sorted so that sv is descending.
// =====================================================================================
namespace {
__device__ __forceinline__ void rr_pair(int np, int r, int i, int &a, int &b) {
    // circle method over np (even) players: player 0 fixed, the rest rotate
    const int m = np - 1;
    if (i == 0) { a = 0; b = (r % m) + 1; }
    else { a = ((r + i) % m) + 1; b = ((r - i + m) % m) + 1; }
}

__global__ void __launch_bounds__(1024) jacobi_kernel(double *W, i64 ldw, double *V, i64 ldv, int n,
                                                      int max_sweeps, int *sweeps_out, int *flag) {
    __shared__ int rotated;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int np = n + (n & 1);
    const double tol = 1e-15;
    int sweep = 0;
    for (; sweep < max_sweeps; sweep++) {
        if (threadIdx.x == 0) rotated = 0;
        __syncthreads();
        for (int r = 0; r < np - 1; r++) {
            for (int pi = wid; pi < np / 2; pi += nw) {
                int p, q;
                rr_pair(np, r, pi, p, q);
                if (p >= n || q >= n) continue;
                if (p > q) { const int t = p; p = q; q = t; }
                double *wp = W + p * ldw, *wq = W + q * ldw;
                double a = 0, b = 0, d = 0;
                for (int i = lane; i < n; i += 32) {
                    const double x = wp[i], y = wq[i];
                    a = fma(x, x, a); b = fma(y, y, b); d = fma(x, y, d);
                }
                a = warp_sum(a); b = warp_sum(b); d = warp_sum(d);
                if (d == 0.0 || fabs(d) <= tol * sqrt(a * b)) continue;
                const double zeta = (b - a) / (2.0 * d);
                const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                const double cs = 1.0 / sqrt(1.0 + t * t), sn = cs * t;
                for (int i = lane; i < n; i += 32) {
                    const double x = wp[i], y = wq[i];
                    wp[i] = cs * x - sn * y;
                    wq[i] = sn * x + cs * y;
                }
                double *vp = V + p * ldv, *vq = V + q * ldv;
                for (int i = lane; i < n; i += 32) {
                    const double x = vp[i], y = vq[i];
                    vp[i] = cs * x - sn * y;
                    vq[i] = sn * x + cs * y;
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

// sv[j] = |W(:,j)|, rank[j] = position of column j in descending order (ties by index)
__global__ void jacobi_finish_kernel(const double *W, i64 ldw, int n, double *sv, int *rank) {
    const int lane = threadIdx.x & 31;
    for (int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); j < n; j += gridDim.x * (blockDim.x >> 5)) {
        double a = 0;
        for (int i = lane; i < n; i += 32) a = fma(W[i + j * ldw], W[i + j * ldw], a);
        a = warp_sum(a);
        if (lane == 0) sv[j] = sqrt(a);
    }
}
__global__ void jacobi_rank_kernel(const double *sv, int n, int *rank) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double v = sv[j];
    int r = 0;
    for (int i = 0; i < n; i++) r += (sv[i] > v) || (sv[i] == v && i < j);
    rank[j] = r;
}
__global__ void jacobi_scatter_kernel(const double *W, i64 ldw, const double *Vin, i64 ldvi, const double *sv,
                                      const int *rank, int n, double *U, i64 ldu, double *V, i64 ldv,
                                      double *sv_sorted) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < (i64)n * n; e += (i64)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        const int r = rank[j];
        const double s = sv[j];
        U[i + (i64)r * ldu] = (s > 0.0) ? W[i + j * ldw] / s : 0.0;
        V[i + (i64)r * ldv] = Vin[i + j * ldvi];
        if (i == 0) sv_sorted[r] = s;
    }
}
}  // namespace

int jacobi_svd(cudaStream_t s, DM<double> G, DM<double> U, DM<double> V, double *d_sv, int *d_flag) {
    const int n = (int)G.r;
    if (G.r != G.c) fail(RSVD_ERR_ARGUMENT, "jacobi: not square");
    if (n == 0) return 0;
    DMat<double> Vacc(n, n, s);
    set_identity(s, Vacc.v);
    DBuf aux(sizeof(int) * (n + 2), s);
    int *d_sweeps = (int *)aux.get();
    int *d_rank = d_sweeps + 2;
    DBuf svbuf(sizeof(double) * n, s);
    double *d_sv_raw = (double *)svbuf.get();
    RSVD_CK(cudaMemsetAsync(d_flag, 0, sizeof(int), s));
    jacobi_kernel<<<1, 1024, 0, s>>>(G.p, G.ld, Vacc.v.p, Vacc.v.ld, n, 60, d_sweeps, d_flag);
    RSVD_LAUNCH_CK();
    jacobi_finish_kernel<<<ceil_div(n, 8), 256, 0, s>>>(G.p, G.ld, n, d_sv_raw, d_rank);
    jacobi_rank_kernel<<<ceil_div(n, 256), 256, 0, s>>>(d_sv_raw, n, d_rank);
    jacobi_scatter_kernel<<<grid_for((i64)n * n), 256, 0, s>>>(G.p, G.ld, Vacc.v.p, Vacc.v.ld, d_sv_raw, d_rank, n,
                                                               U.p, U.ld, V.p, V.ld, d_sv);
    RSVD_LAUNCH_CK();
    int sweeps = 0;
    RSVD_CK(cudaMemcpyAsync(&sweeps, d_sweeps, sizeof(int), cudaMemcpyDeviceToHost, s));
    RSVD_CK(cudaStreamSynchronize(s));
    return sweeps;
}

// =====================================================================================
// Householder QR (fallback when CholeskyQR breaks down): LAPACK-style reflectors
// H = I - tau v v^T with v(0) = 1, beta = -sign(alpha) |x|.
// =====================================================================================
namespace {
template <typename T>
__global__ void hh_make_kernel(T *Y, i64 ld, i64 m, int j, double *tau, double *R, i64 ldr) {
    __shared__ double sc[32];
    double sig = 0.0;
    for (i64 i = j + 1 + threadIdx.x; i < m; i += blockDim.x) {
        const double v = (double)Y[i + j * ld];
        sig = fma(v, v, sig);
    }
    sig = block_sum(sig, sc);
    const double alpha = (double)Y[j + j * ld];
    double beta, t, scale;
    if (sig == 0.0) { t = 0.0; beta = alpha; scale = 0.0; }
    else {
        const double nrm = sqrt(alpha * alpha + sig);
        beta = (alpha >= 0.0) ? -nrm : nrm;
        t = (beta - alpha) / beta;
        scale = 1.0 / (alpha - beta);
    }
    for (i64 i = j + 1 + threadIdx.x; i < m; i += blockDim.x) Y[i + j * ld] = (T)((double)Y[i + j * ld] * scale);
    if (threadIdx.x == 0) {
        tau[j] = t;
        R[j + (i64)j * ldr] = beta;
    }
}
// apply H_j from the left to columns [c0, c1) of X (rows j..m-1), reflector in column j of V
template <typename T>
__global__ void hh_apply_kernel(const T *V, i64 ldv, T *X, i64 ldx, i64 m, int j, int c0, const double *tau) {
    __shared__ double sc[32];
    const int col = c0 + blockIdx.x;
    const double t = tau[j];
    if (t == 0.0) return;
    T *x = X + (i64)col * ldx;
    const T *v = V + (i64)j * ldv;
    double w = (double)x[j];
    double part = 0.0;
    for (i64 i = j + 1 + threadIdx.x; i < m; i += blockDim.x) part = fma((double)v[i], (double)x[i], part);
    w += block_sum(part, sc);
    const double f = t * w;
    if (threadIdx.x == 0) x[j] = (T)((double)x[j] - f);
    for (i64 i = j + 1 + threadIdx.x; i < m; i += blockDim.x) x[i] = (T)((double)x[i] - f * (double)v[i]);
}
template <typename T>
__global__ void hh_copy_r_kernel(const T *Y, i64 ld, int c, double *R, i64 ldr) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < c * c; e += gridDim.x * blockDim.x) {
        const int i = e % c, k = e / c;
        if (i < k) R[i + (i64)k * ldr] = (double)Y[i + (i64)k * ld];
        else if (i > k) R[i + (i64)k * ldr] = 0.0;
    }
}
}  // namespace

template <typename T>
void householder_qr(cudaStream_t s, DM<T> Y, DM<T> Q, DM<double> R) {
    const i64 m = Y.r;
    const int c = (int)Y.c;
    if (m < c) fail(RSVD_ERR_ARGUMENT, "householder_qr: needs rows >= cols");
    DBuf taub(sizeof(double) * std::max(1, c), s);
    double *tau = (double *)taub.get();
    for (int j = 0; j < c; j++) {
        hh_make_kernel<T><<<1, 256, 0, s>>>(Y.p, Y.ld, m, j, tau, R.p, R.ld);
        if (j + 1 < c) hh_apply_kernel<T><<<c - j - 1, 256, 0, s>>>(Y.p, Y.ld, Y.p, Y.ld, m, j, j + 1, tau);
    }
    hh_copy_r_kernel<T><<<ceil_div((i64)c * c, 256), 256, 0, s>>>(Y.p, Y.ld, c, R.p, R.ld);
    set_identity(s, Q);
    for (int j = c - 1; j >= 0; j--)
        hh_apply_kernel<T><<<c - j, 256, 0, s>>>(Y.p, Y.ld, Q.p, Q.ld, m, j, j, tau);
    RSVD_LAUNCH_CK();
}
template void householder_qr<double>(cudaStream_t, DM<double>, DM<double>, DM<double>);
template void householder_qr<float>(cudaStream_t, DM<float>, DM<float>, DM<double>);

// =====================================================================================
// Gram G = Y^T Y (FP64 result).  32x32 tile of G per block, rows of Y split into
// 2048-row slabs over blockIdx.z; per-slab partials are reduced in a fixed order
// (deterministic).  float data: FP32 products/sums over 256 rows, then FP64.
// =====================================================================================
namespace {
constexpr int GR_SLAB = 2048;
template <typename T>
__global__ void __launch_bounds__(256) gram_kernel(const T *__restrict__ Y, i64 ld, i64 m, int c,
                                                   double *__restrict__ part, i64 part_stride) {
    __shared__ T Ya[32][33];
    __shared__ T Yb[32][33];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
    const i64 r0 = (i64)blockIdx.z * GR_SLAB, r1 = min(m, r0 + GR_SLAB);
    double dacc[2][2] = {{0, 0}, {0, 0}};
    T acc[2][2] = {{T(0), T(0)}, {T(0), T(0)}};
    int since = 0;
    for (i64 rb = r0; rb < r1; rb += 32) {
        for (int e = threadIdx.x; e < 32 * 32; e += 256) {
            const int rr = e & 31, cc = e >> 5;
            const i64 row = rb + rr;
            Ya[rr][cc] = (row < r1 && i0 + cc < c) ? Y[row + (i64)(i0 + cc) * ld] : T(0);
            Yb[rr][cc] = (row < r1 && j0 + cc < c) ? Y[row + (i64)(j0 + cc) * ld] : T(0);
        }
        __syncthreads();
#pragma unroll 8
        for (int rr = 0; rr < 32; rr++) {
            const T a0 = Ya[rr][ty], a1 = Ya[rr][ty + 16];
            const T b0 = Yb[rr][tx], b1 = Yb[rr][tx + 16];
            acc[0][0] = fma(a0, b0, acc[0][0]);
            acc[0][1] = fma(a0, b1, acc[0][1]);
            acc[1][0] = fma(a1, b0, acc[1][0]);
            acc[1][1] = fma(a1, b1, acc[1][1]);
        }
        __syncthreads();
        if (++since == 8) {
#pragma unroll
            for (int x = 0; x < 2; x++)
#pragma unroll
                for (int y = 0; y < 2; y++) { dacc[x][y] += (double)acc[x][y]; acc[x][y] = T(0); }
            since = 0;
        }
    }
#pragma unroll
    for (int x = 0; x < 2; x++)
#pragma unroll
        for (int y = 0; y < 2; y++) {
            dacc[x][y] += (double)acc[x][y];
            const int gi = i0 + ty + 16 * x, gj = j0 + tx + 16 * y;
            if (gi < c && gj < c) part[(i64)blockIdx.z * part_stride + gi + (i64)gj * c] = dacc[x][y];
        }
}
__global__ void gram_reduce_kernel(const double *part, i64 part_stride, int nslab, int c, double *G, i64 ldg) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < (i64)c * c; e += (i64)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int z = 0; z < nslab; z++) acc += part[z * part_stride + e];
        G[(e % c) + (e / c) * ldg] = acc;
    }
}
// Reduce into FP32 packed upper 32 x 32 tiles (tile (I, K), I <= K, at (K(K+1)/2 + I) *
// 1024, row-major), padded to np = 32 * ceil(c / 32) with the identity; optionally also
// into the full symmetric FP64 G.
__global__ void gram_reduce_tiles_kernel(const double *part, i64 part_stride, int nslab, int c, int np, float *Gt,
                                         double *G, i64 ldg) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < np * np; e += gridDim.x * blockDim.x) {
        const int i = e % np, j = e / np;
        if (i > j) continue;
        double v;
        if (i < c && j < c) {
            v = 0.0;
            for (int z = 0; z < nslab; z++) v += part[z * part_stride + i + (i64)j * c];
            if (G) {
                G[i + (i64)j * ldg] = v;
                G[j + (i64)i * ldg] = v;
            }
        } else {
            v = (i == j) ? 1.0 : 0.0;
        }
        const int I = i >> 5, K = j >> 5;
        Gt[(size_t)(K * (K + 1) / 2 + I) * 1024 + (i & 31) * 32 + (j & 31)] = (float)v;
    }
}
}  // namespace

// FP32 Gram, symmetric tiles only: 64 x 64 tile (bi <= bj) of G per block over a 1024-row
// slab, 256 threads with 4 x 4 outputs each, FP32 sums flushed to FP64 every 256 rows.
// Off-diagonal tiles are written to both (bi,bj) and (bj,bi) of the slab partial.
namespace {
constexpr int GS_SLAB = 1024;
__global__ void __launch_bounds__(256) gram_sym_f32_kernel(const float *__restrict__ Y, i64 ld, i64 m, int c,
                                                           int ntile, double *__restrict__ part, i64 part_stride) {
    // column-major staging tiles [column][row], pitch 33: the staging stores (32 rows of
    // one column per warp) and the compute loads (16 distinct columns per warp) are
    // free of bank conflicts
    __shared__ float As[64][33];
    __shared__ float Bs[64][33];
    // upper-triangular tile list: blockIdx.x -> (bi, bj), bi <= bj
    int bj = 0;
    while ((bj + 1) * (bj + 2) / 2 <= (int)blockIdx.x) bj++;
    const int bi = (int)blockIdx.x - bj * (bj + 1) / 2;
    const int i0 = bi * 64, j0 = bj * 64;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const i64 r0 = (i64)blockIdx.y * GS_SLAB, r1 = min(m, r0 + GS_SLAB);
    float acc[4][4];
    double dacc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) { acc[a][b] = 0.f; dacc[a][b] = 0.0; }
    int since = 0;
    for (i64 rb = r0; rb < r1; rb += 32) {
#pragma unroll
        for (int e = 0; e < 8; e++) {
            const int idx = tid + 256 * e;
            const int kk = idx & 31, cc = idx >> 5;
            const i64 row = rb + kk;
            As[cc][kk] = (row < r1 && i0 + cc < c) ? Y[row + (i64)(i0 + cc) * ld] : 0.f;
            Bs[cc][kk] = (row < r1 && j0 + cc < c) ? Y[row + (i64)(j0 + cc) * ld] : 0.f;
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < 32; kk++) {
            float av[4], bv[4];
#pragma unroll
            for (int x = 0; x < 4; x++) av[x] = As[ty + 16 * x][kk];
#pragma unroll
            for (int y = 0; y < 4; y++) bv[y] = Bs[tx + 16 * y][kk];
#pragma unroll
            for (int x = 0; x < 4; x++)
#pragma unroll
                for (int y = 0; y < 4; y++) acc[x][y] = fmaf(av[x], bv[y], acc[x][y]);
        }
        __syncthreads();
        if (++since == 8) {
#pragma unroll
            for (int x = 0; x < 4; x++)
#pragma unroll
                for (int y = 0; y < 4; y++) { dacc[x][y] += (double)acc[x][y]; acc[x][y] = 0.f; }
            since = 0;
        }
    }
    double *P = part + (i64)blockIdx.y * part_stride;
#pragma unroll
    for (int x = 0; x < 4; x++)
#pragma unroll
        for (int y = 0; y < 4; y++) {
            const double v = dacc[x][y] + (double)acc[x][y];
            const int gi = i0 + ty + 16 * x, gj = j0 + tx + 16 * y;
            if (gi < c && gj < c) {
                P[gi + (i64)gj * c] = v;
                if (bi != bj) P[gj + (i64)gi * c] = v;
            }
        }
    (void)ntile;
}
}  // namespace

template <typename T>
void gram(cudaStream_t s, DM<T> Y, DM<double> G) {
    const int c = (int)Y.c;
    if (G.r != c || G.c != c) fail(RSVD_ERR_ARGUMENT, "gram: shape mismatch");
    if (c == 0) return;
    if (std::is_same<T, float>::value && c >= 64) {
        const int nt = (c + 63) / 64, ntiles = nt * (nt + 1) / 2;
        const int nslab = (int)std::max<i64>(1, (Y.r + GS_SLAB - 1) / GS_SLAB);
        const i64 stride = (i64)c * c;
        if (nslab <= 65535) {
            DBuf part(sizeof(double) * (size_t)stride * nslab, s);
            gram_sym_f32_kernel<<<dim3(ntiles, nslab), 256, 0, s>>>((const float *)Y.p, Y.ld, Y.r, c, ntiles,
                                                                    (double *)part.get(), stride);
            gram_reduce_kernel<<<grid_for(stride), 256, 0, s>>>((const double *)part.get(), stride, nslab, c, G.p,
                                                                G.ld);
            RSVD_LAUNCH_CK();
            ctx().launches += 2;
            return;
        }
    }
    const int nslab = (int)std::max<i64>(1, (Y.r + GR_SLAB - 1) / GR_SLAB);
    const i64 stride = (i64)c * c;
    DBuf part(sizeof(double) * (size_t)stride * nslab, s);
    dim3 grid(ceil_div(c, 32), ceil_div(c, 32), nslab);
    gram_kernel<T><<<grid, 256, 0, s>>>(Y.p, Y.ld, Y.r, c, (double *)part.get(), stride);
    gram_reduce_kernel<<<grid_for(stride), 256, 0, s>>>((const double *)part.get(), stride, nslab, c, G.p, G.ld);
    RSVD_LAUNCH_CK();
    ctx().launches += 2;
}
template void gram<double>(cudaStream_t, DM<double>, DM<double>);
template void gram<float>(cudaStream_t, DM<float>, DM<double>);

namespace {
// Dense FP32 c x c Gram (upper triangle read) -> packed upper 32 x 32 tiles (identity
// padding), and optionally both halves of the FP64 copy.
__global__ void pack_gram_tiles_kernel(const float *Gd, i64 ldd, int c, int np, float *Gt, double *G, i64 ldg) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < np * np; e += gridDim.x * blockDim.x) {
        const int i = e % np, j = e / np;
        if (i > j) continue;
        float v;
        if (i < c && j < c) {
            v = Gd[i + (i64)j * ldd];
            if (G) {
                G[i + (i64)j * ldg] = (double)v;
                G[j + (i64)i * ldg] = (double)v;
            }
        } else {
            v = (i == j) ? 1.f : 0.f;
        }
        const int I = i >> 5, K = j >> 5;
        Gt[(size_t)(K * (K + 1) / 2 + I) * 1024 + (i & 31) * 32 + (j & 31)] = v;
    }
}
}  // namespace

void gram_tiles_f32(cudaStream_t s, DM<float> Y, float *Gt, DM<double> *G) {
    const int c = (int)Y.c;
    if (c == 0) return;
    if (G && (G->r != c || G->c != c)) fail(RSVD_ERR_ARGUMENT, "gram: shape mismatch");
    const int prec = ctx().opts.precision;
    if ((prec == RSVD_PREC_TF32 || prec == RSVD_PREC_BF16) && Y.r >= 2048 && c >= 64) {
        // tensor-core modes: G = Y^T Y by 3xTF32 (FP32-accurate) as ONE split-K launch of the
        // three terms lo x hi, hi x lo, hi x hi (chains of m / 64 k-blocks across the concatenated
        // terms, compensated sums across chains); two launches, their reductions and an add
        // cost twice as much at m = 16384
        const int np = (c + 31) / 32 * 32;
        DMat<float> Yh(Y.r, c, s, false), Yl(Y.r, c, s, false), Gd(c, c, s, false);
        split_tf32(s, Y.p, Y.ld, Y.r, c, Yh.v.p, Yl.v.p, Yh.v.ld);
        const int m = (int)Y.r;
        const TcSeg sg[3] = {{Yl.v.p, Yl.v.ld, Yh.v.p, Yh.v.ld, m}, {Yh.v.p, Yh.v.ld, Yl.v.p, Yl.v.ld, m},
                             {Yh.v.p, Yh.v.ld, Yh.v.p, Yh.v.ld, m}};
        const int splits = std::max(1, std::min(64, m / 256));
        tc_gemm_segs(s, 0 /* kind::tf32 */, false, 3, sg, c, c, 1.0f, Gd.v.p, Gd.v.ld, 0 /* store */, nullptr, 0, nullptr,
                     splits, nullptr);
        pack_gram_tiles_kernel<<<grid_for((i64)np * np), 256, 0, s>>>(Gd.v.p, Gd.v.ld, c, np, Gt, G ? G->p : nullptr,
                                                                     G ? G->ld : 0);
        RSVD_LAUNCH_CK();
        ctx().launches++;
        return;                                 // temporaries are freed in stream order
    }
    const int np = (c + 31) / 32 * 32;
    const i64 stride = (i64)c * c;
    int nslab;
    DBuf part;
    if (c >= 64 && (Y.r + GS_SLAB - 1) / GS_SLAB <= 65535) {
        const int nt = (c + 63) / 64, ntiles = nt * (nt + 1) / 2;
        nslab = (int)std::max<i64>(1, (Y.r + GS_SLAB - 1) / GS_SLAB);
        part = DBuf(sizeof(double) * (size_t)stride * nslab, s);
        gram_sym_f32_kernel<<<dim3(ntiles, nslab), 256, 0, s>>>(Y.p, Y.ld, Y.r, c, ntiles, (double *)part.get(), stride);
    } else {
        nslab = (int)std::max<i64>(1, (Y.r + GR_SLAB - 1) / GR_SLAB);
        part = DBuf(sizeof(double) * (size_t)stride * nslab, s);
        dim3 grid(ceil_div(c, 32), ceil_div(c, 32), nslab);
        gram_kernel<float><<<grid, 256, 0, s>>>(Y.p, Y.ld, Y.r, c, (double *)part.get(), stride);
    }
    gram_reduce_tiles_kernel<<<grid_for((i64)np * np), 256, 0, s>>>((const double *)part.get(), stride, nslab, c, np,
                                                                     Gt, G ? G->p : nullptr, G ? G->ld : 0);
    RSVD_LAUNCH_CK();
    ctx().launches += 2;
}

}  // namespace rsvd
