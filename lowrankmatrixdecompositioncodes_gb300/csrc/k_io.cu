// k_io.cu -- streaming load of the reference's binary matrix files straight into device memory.
//
// File format (matrix_load_from_binary_file, matrix_vector_functions_intel_mkl.c:77-133; the
// 64-bit and oneAPI variants widen the header to int64 and the oneAPI one stores floats): two
// header integers (rows m, columns n), then the m x n entries row by row.  The host loader of the
// C API reads that into a column-major host `mat`; this path instead reads the file in chunks of
// whole rows into two pinned staging buffers and, per chunk, copies it to the device on a copy
// stream and transposes it there into the caller's column-major device matrix (leading dimension
// lda), converting to FP64, FP32 or BF16 on the way.  Reading chunk c + 1 from the file, copying
// chunk c and transposing chunk c - 1 overlap.
#include "rsvd_internal.h"
#include "k_common.cuh"

#include <cuda_bf16.h>

#include <cstdio>
#include <cstring>
#include <string>

namespace rsvd {

namespace {

template <typename D, typename S>
__device__ __forceinline__ D io_cast(S v);
template <> __device__ __forceinline__ double io_cast<double, double>(double v) { return v; }
template <> __device__ __forceinline__ double io_cast<double, float>(float v) { return (double)v; }
template <> __device__ __forceinline__ float io_cast<float, double>(double v) { return __double2float_rn(v); }
template <> __device__ __forceinline__ float io_cast<float, float>(float v) { return v; }
// FP64 -> BF16 in one rounding: FP64 -> FP32 rounded to odd (truncate, then set the last bit if
// anything was cut off), then FP32 -> BF16 to nearest; with 16 bits to spare in FP32 the odd
// intermediate never creates a false tie, so the result is FP64 rounded to nearest BF16.
template <> __device__ __forceinline__ __nv_bfloat16 io_cast<__nv_bfloat16, double>(double v) {
    float f = __double2float_rz(v);
    if ((double)f != v && isfinite(f)) f = __uint_as_float(__float_as_uint(f) | 1u);
    return __float2bfloat16_rn(f);
}
template <> __device__ __forceinline__ __nv_bfloat16 io_cast<__nv_bfloat16, float>(float v) {
    return __float2bfloat16_rn(v);
}

// A chunk of nr rows (row-major, n per row) -> rows [row0, row0 + nr) of the column-major dst,
// through a 32 x 32 shared-memory tile so that both the reads (along a row) and the writes
// (along a column) are coalesced.  Block 32 x 8.
template <typename S, typename D>
__global__ void rows_to_cols_kernel(const S *__restrict__ src, int nr, int n, D *__restrict__ dst, long long lda,
                                    long long row0) {
    __shared__ S tile[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
    for (int k = 0; k < 32; k += 8) {
        const int r = r0 + ty + k, c = c0 + tx;
        if (r < nr && c < n) tile[ty + k][tx] = src[(size_t)r * n + c];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 32; k += 8) {
        const int c = c0 + ty + k, r = r0 + tx;
        if (r < nr && c < n) dst[row0 + r + (long long)c * lda] = io_cast<D, S>(tile[tx][ty + k]);
    }
}

template <typename S>
void launch_rows_to_cols(cudaStream_t s, const void *src, int nr, int n, int dtype, void *dst, long long lda,
                         long long row0) {
    const dim3 grid((unsigned)((n + 31) / 32), (unsigned)((nr + 31) / 32)), block(32, 8);
    if (dtype == RSVD_DT_F64)
        rows_to_cols_kernel<S, double><<<grid, block, 0, s>>>((const S *)src, nr, n, (double *)dst, lda, row0);
    else if (dtype == RSVD_DT_F32)
        rows_to_cols_kernel<S, float><<<grid, block, 0, s>>>((const S *)src, nr, n, (float *)dst, lda, row0);
    else
        rows_to_cols_kernel<S, __nv_bfloat16><<<grid, block, 0, s>>>((const S *)src, nr, n, (__nv_bfloat16 *)dst, lda,
                                                                     row0);
    RSVD_LAUNCH_CK();
}

struct FileCloser {
    FILE *fp;
    ~FileCloser() {
        if (fp) std::fclose(fp);
    }
};

}  // namespace

bool binary_file_shape(const char *fname, int hdr_bytes, long long *m, long long *n) {
    FILE *fp = std::fopen(fname, "rb");
    if (!fp) return false;
    FileCloser fc{fp};
    if (hdr_bytes == 4) {
        int h[2];
        if (std::fread(h, 4, 2, fp) != 2) return false;
        *m = h[0];
        *n = h[1];
    } else {
        long long h[2];
        if (std::fread(h, 8, 2, fp) != 2) return false;
        *m = h[0];
        *n = h[1];
    }
    return *m > 0 && *n > 0;
}

void load_binary_to_device(const char *fname, int hdr_bytes, int real_bytes, int dtype, void *dA, long long lda,
                           long long *m_out, long long *n_out) {
    Ctx &cx = ctx();
    cudaStream_t s = cx.stream;
    long long m = 0, n = 0;
    if (!binary_file_shape(fname, hdr_bytes, &m, &n))
        fail(RSVD_ERR_ARGUMENT, std::string("cannot read a matrix file header from ") + fname);
    if (n > (1ll << 30)) fail(RSVD_ERR_ARGUMENT, "matrix file: too many columns");
    if (lda < m) fail(RSVD_ERR_ARGUMENT, "leading dimension below the file's row count");
    FILE *fp = std::fopen(fname, "rb");
    if (!fp) fail(RSVD_ERR_ARGUMENT, std::string("cannot open ") + fname);
    FileCloser fc{fp};
    if (std::fseek(fp, 2L * hdr_bytes, SEEK_SET) != 0) fail(RSVD_ERR_ARGUMENT, "matrix file: seek failed");
    // chunks of whole rows, ~32 MiB each
    const size_t row_bytes = (size_t)n * (size_t)real_bytes;
    const long long rows_per = std::max<long long>(1, std::min<long long>(m, (32ll << 20) / (long long)row_bytes));
    const size_t chunk_bytes = (size_t)rows_per * row_bytes;
    void *hbuf[2] = {nullptr, nullptr};
    cudaStream_t cs = nullptr;
    cudaEvent_t copied[2] = {nullptr, nullptr}, consumed[2] = {nullptr, nullptr};
    DBuf dbuf[2] = {DBuf(chunk_bytes, s), DBuf(chunk_bytes, s)};
    auto cleanup = [&] {
        for (int b = 0; b < 2; b++) {
            if (copied[b]) cudaEventDestroy(copied[b]);
            if (consumed[b]) cudaEventDestroy(consumed[b]);
            if (hbuf[b]) cudaFreeHost(hbuf[b]);
        }
        if (cs) cudaStreamDestroy(cs);
    };
    try {
        for (int b = 0; b < 2; b++) {
            RSVD_CK(cudaHostAlloc(&hbuf[b], chunk_bytes, cudaHostAllocDefault));
            RSVD_CK(cudaEventCreateWithFlags(&copied[b], cudaEventDisableTiming));
            RSVD_CK(cudaEventCreateWithFlags(&consumed[b], cudaEventDisableTiming));
        }
        RSVD_CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        RSVD_CK(cudaStreamSynchronize(s));       // the staging buffers' allocation is ordered before cs uses them
        long long row0 = 0;
        for (int c = 0; row0 < m; c++) {
            const int b = c & 1;
            const long long nr = std::min(rows_per, m - row0);
            // the pinned buffer is free once the transpose that read its previous contents has run
            if (c >= 2) RSVD_CK(cudaEventSynchronize(consumed[b]));
            const size_t bytes = (size_t)nr * row_bytes;
            if (std::fread(hbuf[b], 1, bytes, fp) != bytes) fail(RSVD_ERR_ARGUMENT, "truncated matrix file");
            RSVD_CK(cudaMemcpyAsync(dbuf[b].get(), hbuf[b], bytes, cudaMemcpyHostToDevice, cs));
            RSVD_CK(cudaEventRecord(copied[b], cs));
            RSVD_CK(cudaStreamWaitEvent(s, copied[b], 0));
            if (real_bytes == 8)
                launch_rows_to_cols<double>(s, dbuf[b].get(), (int)nr, (int)n, dtype, dA, lda, row0);
            else
                launch_rows_to_cols<float>(s, dbuf[b].get(), (int)nr, (int)n, dtype, dA, lda, row0);
            ctx().launches++;
            RSVD_CK(cudaEventRecord(consumed[b], s));
            row0 += nr;
        }
        RSVD_CK(cudaStreamSynchronize(s));
    } catch (...) {
        cudaStreamSynchronize(s);                 // no copy or transpose may still use the buffers
        if (cs) cudaStreamSynchronize(cs);
        cleanup();
        throw;
    }
    cleanup();
    *m_out = m;
    *n_out = n;
}

}  // namespace rsvd
