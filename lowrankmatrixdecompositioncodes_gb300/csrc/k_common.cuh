// k_common.cuh -- small device helpers shared by the kernel translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace rsvd {

// Status words in Ctx::d_flags (one int each).
enum : int {
    FLAG_CHOL_BREAKDOWN = 0,   // Cholesky met a non-positive pivot
    FLAG_TIMEOUT = 1,          // a bounded wait in a tcgen05 kernel gave up
    FLAG_NONFINITE = 2,        // non-finite value met where it must not be
    FLAG_JACOBI_NOCONV = 3,    // Jacobi hit its sweep limit
    FLAG_COUNT = 8
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum for blockDim.x a multiple of 32 (<= 1024).  All threads get the result.
template <typename T>
__device__ T block_sum(T v, T *scratch32) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) scratch32[wid] = v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    T t = (threadIdx.x < nw) ? scratch32[threadIdx.x] : T(0);
    if (wid == 0) t = warp_sum(t);
    if (threadIdx.x == 0) scratch32[0] = t;
    __syncthreads();
    T r = scratch32[0];
    __syncthreads();
    return r;
}

inline unsigned ceil_div(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace rsvd
