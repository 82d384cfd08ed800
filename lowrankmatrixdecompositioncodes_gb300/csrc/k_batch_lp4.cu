// k_batch_lp4.cu -- the batched rSVD kernel with 4 lanes per Jacobi pair (one instantiation per
// file: the four compile in parallel).
#include "k_batch_dev.cuh"

namespace rsvd {

void batch_rsvd_launch_lp4(cudaStream_t s, const BatchItem *d_items, int count, int *d_queue, float *d_work,
                          long long slab, long long ldw, unsigned long long seed, int q, int s_, int *d_flag, int nctas,
                          size_t smem, int cuadd) {
    batch_rsvd_launch_impl<4>(s, d_items, count, d_queue, d_work, slab, ldw, seed, q, s_, d_flag, nctas, smem, cuadd);
}

}  // namespace rsvd
