// k_resid.cu -- residual norms of a low-rank approximation: ||A - U diag(S) V^T|| in the Frobenius
// and spectral norms, on the device.
//
// The reference reports only the Frobenius error, by forming the product matrix on the host
// (multi_core_mkl_code/matrix_vector_functions_intel_mkl.c:391-405 get_percent_error_between_two_mats,
// :1304-1318 form_svd_product_matrix).  Here the residual R = A - (U S) V^T is formed once on the
// device -- for FP64 data with the double-float product (k_df64.cu), so that a residual far below
// ||A|| keeps its digits -- and stored in FP32 (its rounding is relative to R's own entries).
//   Frobenius: the sum of squares of R in FP64 (sumsq kernel).
//   Spectral : block power iteration on R^T R (b = 8 vectors, Philox start, orthonormalised every
//              round), then the Rayleigh-Ritz value: the largest singular value of R X for the
//              final orthonormal X.  It approaches ||R||_2 from below; the gap ratio of R's top
//              singular values sets how fast.
#include "engine.h"
#include "k_common.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace rsvd {

namespace {

template <typename T>
__global__ void scale_cols_kernel(const T *U, i64 ldu, const double *S, i64 m, i64 k, T *out, i64 ldo) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < m * k; e += (i64)gridDim.x * blockDim.x) {
        const i64 j = e / m, i = e - j * m;
        out[i + j * ldo] = (T)((double)U[i + j * ldu] * S[j]);
    }
}

unsigned gfor(i64 n) {
    const i64 g = (n + 255) / 256;
    return (unsigned)std::max<i64>(1, std::min<i64>(g, (i64)std::max(1, ctx().sms) * 8));
}

// largest eigenvalue of a small symmetric matrix (host, cyclic Jacobi in FP64)
double sym_eig_max(std::vector<double> a, int n) {
    for (int sweep = 0; sweep < 50; sweep++) {
        double off = 0.0;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) off += a[p + q * n] * a[p + q * n];
        if (off < 1e-30) break;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) {
                const double apq = a[p + q * n];
                if (apq == 0.0) continue;
                const double zeta = (a[q + q * n] - a[p + p * n]) / (2.0 * apq);
                const double t = std::copysign(1.0, zeta) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
                const double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
                for (int r = 0; r < n; r++) {     // columns p, q
                    const double x = a[r + p * n], y = a[r + q * n];
                    a[r + p * n] = c * x - s * y;
                    a[r + q * n] = s * x + c * y;
                }
                for (int r = 0; r < n; r++) {     // rows p, q
                    const double x = a[p + r * n], y = a[q + r * n];
                    a[p + r * n] = c * x - s * y;
                    a[q + r * n] = s * x + c * y;
                }
            }
    }
    double mx = 0.0;
    for (int i = 0; i < n; i++) mx = std::max(mx, a[i + i * n]);
    return mx;
}

}  // namespace

template <typename T>
void residual_norms(DM<T> A, DM<T> U, const double *dS, DM<T> V, double *fro, double *spec, int iters) {
    Ctx &cx = ctx();
    cudaStream_t s = cx.stream;
    const i64 m = A.r, n = A.c, k = U.c;
    if (U.r != m || V.r != n || V.c != k) fail(RSVD_ERR_ARGUMENT, "residual_norms: shapes");
    // R = A - (U S) V^T, stored FP32
    DMat<float> R(m, n, s, false);
    if (k == 0) {
        convert<T, float>(s, A, R.v);
    } else {
        DMat<T> US(m, k, s, false);
        scale_cols_kernel<T><<<gfor(m * k), 256, 0, s>>>(U.p, U.ld, dS, m, k, US.v.p, US.v.ld);
        RSVD_LAUNCH_CK();
        if constexpr (std::is_same<T, double>::value) {
            DMat<double> R64(m, n, s, false);
            convert<double, double>(s, A, R64.v);
            Df64Split us(s, US.v), vs(s, V);
            df64_gemm(s, false, true, -1.0, us, vs, 1.0, R64.v);
            convert<double, float>(s, R64.v, R.v);
        } else {
            DMat<float> Vt(k, n, s, false);
            transpose<float>(s, V, Vt.v);
            convert<float, float>(s, A, R.v);
            gemm<float>(s, false, false, -1.f, US.v, Vt.v, 1.f, R.v);
        }
    }
    if (fro) *fro = frob_norm<float>(s, R.v);
    if (!spec) return;
    const i64 b = std::min<i64>(8, std::min(m, n));
    if (b <= 0) {
        *spec = 0.0;
        return;
    }
    DMat<float> X(n, b, s, false), Xo(n, b, s, false), Y(m, b, s, false);
    philox_gaussian(s, 0x5EC7A1ull, 0, X.v);
    DM<float> x = X.v;
    for (int it = 0; it < iters; it++) {
        gemm<float>(s, false, false, 1.f, R.v, x, 0.f, Y.v);              // Y = R X
        gemm<float>(s, true, false, 1.f, R.v, Y.v, 0.f, X.v);             // X = R^T Y
        orth<float>(X.v, Xo.v, nullptr, 1);
        x = Xo.v;
    }
    gemm<float>(s, false, false, 1.f, R.v, x, 0.f, Y.v);
    // G = Y^T Y in FP64 on the host (b x b)
    std::vector<float> hy((size_t)(m * b));
    RSVD_CK(cudaMemcpy2DAsync(hy.data(), sizeof(float) * m, Y.v.p, sizeof(float) * Y.v.ld, sizeof(float) * m, b,
                              cudaMemcpyDeviceToHost, s));
    RSVD_CK(cudaStreamSynchronize(s));
    std::vector<double> g((size_t)(b * b), 0.0);
    for (i64 p = 0; p < b; p++)
        for (i64 q = p; q < b; q++) {
            double acc = 0.0;
            for (i64 i = 0; i < m; i++) acc += (double)hy[i + p * m] * (double)hy[i + q * m];
            g[p + q * b] = g[q + p * b] = acc;
        }
    *spec = std::sqrt(std::max(0.0, sym_eig_max(g, (int)b)));
}
template void residual_norms<double>(DM<double>, DM<double>, const double *, DM<double>, double *, double *, int);
template void residual_norms<float>(DM<float>, DM<float>, const double *, DM<float>, double *, double *, int);

}  // namespace rsvd
