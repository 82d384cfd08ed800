// k_batch.h -- shared declarations of the batched fixed-rank rSVD (k_batch.cu: plans, autotuner,
// C ABI; k_batch_dev.cuh: the persistent kernel; k_batch_lp*.cu: one instantiation each, so that
// the four compile in parallel).
#pragma once
#include "rsvd_internal.h"

#include <cstddef>
#include <cstdint>

namespace rsvd {

struct BatchItem {
    const float *A;
    long long lda;
    float *U;
    long long ldu;
    double *S;
    float *V;
    long long ldv;
    int m, n, k, l;
    int index;     // position in the caller's batch (Philox stream offset)
    int pad;
};

constexpr int BT = 256;          // threads per CTA
constexpr int ATP = 68;          // pitch of a staged A chunk (64 values + 4, 16-byte rows)

// The persistent kernel with LP lanes per Jacobi pair (LP in {4, 8, 16, 32}), launched on nctas CTAs.
void batch_rsvd_launch_lp4(cudaStream_t s, const BatchItem *d_items, int count, int *d_queue, float *d_work,
                           long long slab, long long ldw, unsigned long long seed, int q, int s_, int *d_flag, int nctas,
                           size_t smem, int cuadd);
void batch_rsvd_launch_lp8(cudaStream_t s, const BatchItem *d_items, int count, int *d_queue, float *d_work,
                           long long slab, long long ldw, unsigned long long seed, int q, int s_, int *d_flag, int nctas,
                           size_t smem, int cuadd);
void batch_rsvd_launch_lp16(cudaStream_t s, const BatchItem *d_items, int count, int *d_queue, float *d_work,
                            long long slab, long long ldw, unsigned long long seed, int q, int s_, int *d_flag,
                            int nctas, size_t smem, int cuadd);
void batch_rsvd_launch_lp32(cudaStream_t s, const BatchItem *d_items, int count, int *d_queue, float *d_work,
                            long long slab, long long ldw, unsigned long long seed, int q, int s_, int *d_flag,
                            int nctas, size_t smem, int cuadd);

}  // namespace rsvd
