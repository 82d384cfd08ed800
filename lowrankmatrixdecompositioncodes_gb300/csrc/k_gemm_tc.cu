// k_gemm_tc.cu -- tensor-core GEMM for sm_103a: TMA -> shared memory (128B swizzle)
// -> tcgen05.mma (kind::tf32 or kind::f16 with bf16 operands) -> TMEM accumulator ->
// tcgen05.ld epilogue.  This carries every large product of the mixed-precision modes:
//   form N : D (m x w) = A X        A column-major: operand A is MN-major (m contiguous)
//   form T : D (n x w) = A^T X      A column-major: operand A is K-major (m contiguous)
//   update : A (m x n) -= Qp Bp     (blocked QB deflation, fused: no m x n temporary)
// In every form the second operand is K-major: X (column-major, K = its rows).
//
// CTA = 128 threads: thread 0 issues TMA loads, thread 32 issues MMAs, warp 2 owns the
// TMEM allocation, all four warps run the epilogue (warp w reads TMEM lanes 32w..32w+31,
// i.e. rows m0+32w..).  One CTA computes a 128-row tile for all N <= 512 columns, so A is
// streamed from HBM exactly once per product; split-K over grid.z (deterministic
// two-phase reduction) raises the CTA count when there are few row tiles.
// Every mbarrier wait is bounded (~1 s); on timeout the kernel sets FLAG_TIMEOUT, skips
// the remaining work, frees its TMEM and returns.
#include "rsvd_internal.h"
#include "k_common.cuh"

#include <cuda.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>

namespace rsvd {
namespace tc {

constexpr int BM = 128;          // UMMA M (cta_group::1): one TMEM lane per output row
constexpr int KB = 128;          // bytes of K per pipeline stage (one 128B swizzle row)
constexpr int NTHR = 128;
constexpr int A_BYTES = BM * KB; // 16 KB per stage for operand A
constexpr int MAX_BN = 512;      // TMEM columns available to one CTA
constexpr int MAX_SEG = 3;       // K segments per product (3xTF32 terms in one accumulation)
constexpr int CW = 64;           // update epilogue: C columns per TMA chunk (128 x 64 FP32 = 32 KB)

enum { KIND_TF32 = 0, KIND_BF16 = 1 };
enum { EPI_STORE = 0, EPI_UPDATE = 1, EPI_PARTIAL = 2 };

struct Params {
    float *D;          // output (or partial workspace base for EPI_PARTIAL)
    long long ldd;
    long long part_stride;   // EPI_PARTIAL: elements between split slabs
    const float *C;    // EPI_UPDATE: D = C - alpha * acc (C may equal D)
    long long ldc;
    int M, N, K;
    int BN;            // columns per CTA (multiple of 16, <= 512)
    int chunk_n0, chunk_n1;   // MMA N of the (up to) two column chunks (chunk_n1 may be 0)
    int kb_per_split;  // K blocks handled by one split
    int num_kb;        // total K blocks (over all segments)
    int nseg;          // K segments: segment s contracts maps.a[s] with maps.b[s] over seg_kb[s] blocks
    int seg_kb[MAX_SEG];
    int c_tma;         // EPI_UPDATE: C is TMA-loaded into the free stage buffers, D TMA-stored
    // EPI_UPDATE with c_tma (optional, null = none): the new D also split as TF32 hi / lo
    // (hi = D rounded to TF32, lo = D - hi; ld lds) and as BF16 hi / lo (ld ldb)
    float *Shi, *Slo;
    __nv_bfloat16 *Bhi, *Blo;
    long long lds, ldb;
    int stages;
    float alpha;
    double *fro_part;  // EPI_UPDATE: per-CTA sum of squares of the new D (or null)
    int *flag;         // FLAG_TIMEOUT word
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up after ~2^31 SM cycles (about one second), or as soon as another
// thread of the CTA has given up.
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag, int *gflag) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (*abort_flag) return false;
        if (clock64() - t0 > (1ll << 31)) {
            *abort_flag = 1;
            atomicExch(gflag, 1);
            return false;
        }
    }
    return true;
}

// Operand maps of the K segments, and the (unswizzled) C / D maps of the update epilogue.
struct Maps {
    CUtensorMap a[MAX_SEG], b[MAX_SEG], c, d;
};

__device__ __forceinline__ void tma_store_2d(const CUtensorMap *tm, uint32_t src, int c0, int c1) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(
                     (unsigned long long)tm),
                 "r"(src), "r"(c0), "r"(c1)
                 : "memory");
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *tm, uint32_t bar, int c0, int c1) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(dst),
        "l"((unsigned long long)tm), "r"(bar), "r"(c0), "r"(c1)
        : "memory");
}

// UMMA shared-memory descriptor, SM100 layout: start>>4 [0,14), LBO>>4 [16,30),
// SBO>>4 [32,46), version 1 at bit 46, layout SWIZZLE_128B (2) at bits [61,64).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Instruction descriptor (kind::tf32 / kind::f16): D f32 (bits 4-5 = 1), A/B format
// (bits 7-9 / 10-12: bf16 = 1, tf32 = 2), A major (bit 15: 1 = MN-major), B K-major,
// N>>3 at bits 17-22, M>>4 at bits 24-28.
__host__ __device__ constexpr uint32_t make_idesc(int kind, bool a_mn, int n) {
    return (1u << 4) | ((kind == KIND_TF32 ? 2u : 1u) << 7) | ((kind == KIND_TF32 ? 2u : 1u) << 10) |
           ((a_mn ? 1u : 0u) << 15) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

template <int KIND>
__device__ __forceinline__ void umma(uint32_t dt, uint64_t ad, uint64_t bd, uint32_t id, uint32_t acc) {
    if (KIND == KIND_TF32)
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dt),
            "l"(ad), "l"(bd), "r"(id), "r"(acc)
            : "memory");
    else
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dt),
            "l"(ad), "l"(bd), "r"(id), "r"(acc)
            : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Kahan-compensated FP32 accumulation (the update epilogue's sum of squares; FP64 per
// element would cost more than the epilogue itself on GB300).
struct KahanF {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c, t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

template <int KIND, bool A_MN, int EPI>
__global__ void __launch_bounds__(NTHR, 1)
    tc_gemm_kernel(const __grid_constant__ Maps maps, Params P) {
    extern __shared__ uint8_t smem_raw[];
    // 1024-byte alignment for the 128B-swizzled tiles
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    uint8_t *sbase = smem_raw + (base - raw);
    const int stages = P.stages;
    const uint32_t b_bytes = (uint32_t)P.BN * KB;
    const uint32_t stage_bytes = A_BYTES + b_bytes;
    uint64_t *bars = (uint64_t *)(sbase + (size_t)stages * stage_bytes);
    uint64_t *full = bars, *empty = bars + stages, *done = bars + 2 * stages;
    uint64_t *cbar = done + 1;                       // update epilogue: one per C chunk (<= 4)
    uint32_t *tmem_holder = (uint32_t *)(cbar + 4);
    volatile int *abort_flag = (volatile int *)(tmem_holder + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * BM;
    const int n0 = blockIdx.y * P.BN;
    const int kb0 = blockIdx.z * P.kb_per_split;
    const int kb1 = min(P.num_kb, kb0 + P.kb_per_split);
    const int nkb = max(0, kb1 - kb0);

    uint32_t ncols = 32;
    while ((int)ncols < P.BN) ncols <<= 1;

    if (threadIdx.x == 0) {
        for (int s = 0; s < stages; s++) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), 1);
        }
        mbar_init(smem_u32(done), 1);
        for (int c = 0; c < 4; c++) mbar_init(smem_u32(&cbar[c]), 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 2) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_holder;

    // K elements per stage and per MMA
    constexpr int ESZ = (KIND == KIND_TF32) ? 4 : 2;
    constexpr int KE = KB / ESZ;                  // 32 (tf32) or 64 (bf16)
    constexpr int ATOM_M = KB / ESZ;              // MN-major: M elements per 128B row
    constexpr int KSTEP = 32 / ESZ;               // K per MMA instruction: 8 (tf32) / 16 (bf16)

    if (threadIdx.x == 0 && nkb > 0) {
        // ---------------- TMA producer
        for (int i = 0; i < nkb; i++) {
            const int s = i % stages;
            const uint32_t ph = (uint32_t)(i / stages) & 1u;
            if (!mbar_wait(smem_u32(&empty[s]), ph ^ 1u, abort_flag, P.flag)) break;
            const uint32_t sa = base + (uint32_t)s * stage_bytes;
            const uint32_t sb = sa + A_BYTES;
            // segment of this K block, and the block's index within it
            int seg = 0, kk = kb0 + i;
            if (P.nseg > 1 && kk >= P.seg_kb[0]) {
                kk -= P.seg_kb[0];
                seg = 1;
                if (P.nseg > 2 && kk >= P.seg_kb[1]) { kk -= P.seg_kb[1]; seg = 2; }
            }
            const CUtensorMap *tmA = &maps.a[seg], *tmB = &maps.b[seg];
            const int kidx = kk * KE;
            uint32_t bytes = 0;
            int nbox_a = 0;
            if (A_MN) {
                for (int j = 0; j < BM / ATOM_M; j++)
                    if (m0 + j * ATOM_M < P.M) { bytes += (uint32_t)ATOM_M * KE * ESZ; nbox_a++; }
            } else {
                bytes += A_BYTES;
            }
            bytes += (uint32_t)P.chunk_n0 * KB;
            if (P.chunk_n1 > 0) bytes += (uint32_t)P.chunk_n1 * KB;
            const uint32_t fb = smem_u32(&full[s]);
            mbar_expect_tx(fb, bytes);
            if (A_MN) {
                for (int j = 0; j < nbox_a; j++)
                    tma_load_2d(sa + (uint32_t)j * (uint32_t)(KE * KB), tmA, fb, m0 + j * ATOM_M, kidx);
            } else {
                tma_load_2d(sa, tmA, fb, kidx, m0);
            }
            tma_load_2d(sb, tmB, fb, kidx, n0);
            if (P.chunk_n1 > 0) tma_load_2d(sb + (uint32_t)P.chunk_n0 * KB, tmB, fb, kidx, n0 + P.chunk_n0);
        }
    } else if (threadIdx.x == 32 && nkb > 0) {
        // ---------------- MMA issuer
        const uint32_t id0 = make_idesc(KIND, A_MN, P.chunk_n0);
        const uint32_t id1 = make_idesc(KIND, A_MN, P.chunk_n1 > 0 ? P.chunk_n1 : 16);
        for (int i = 0; i < nkb; i++) {
            const int s = i % stages;
            const uint32_t ph = (uint32_t)(i / stages) & 1u;
            if (!mbar_wait(smem_u32(&full[s]), ph, abort_flag, P.flag)) break;
            tc_fence_after();
            const uint32_t sa = base + (uint32_t)s * stage_bytes;
            const uint32_t sb = sa + A_BYTES;
#pragma unroll
            for (int ks = 0; ks < KB / 32; ks++) {
                uint64_t ad;
                if (A_MN) ad = sdesc(sa + (uint32_t)ks * (uint32_t)(KSTEP * KB), (uint32_t)(KE * KB), 1024u);
                else ad = sdesc(sa + (uint32_t)ks * 32u, 16u, 1024u);
                const uint32_t acc = (i > 0 || ks > 0) ? 1u : 0u;
                umma<KIND>(tmem, ad, sdesc(sb + (uint32_t)ks * 32u, 16u, 1024u), id0, acc);
                if (P.chunk_n1 > 0)
                    umma<KIND>(tmem + (uint32_t)P.chunk_n0, ad,
                               sdesc(sb + (uint32_t)P.chunk_n0 * KB + (uint32_t)ks * 32u, 16u, 1024u), id1, acc);
            }
            umma_commit(smem_u32(&empty[s]));
        }
        umma_commit(smem_u32(done));
    }
    __syncwarp();

    // ---------------- epilogue: TMEM -> registers -> global
    bool ok = true;
    if (nkb > 0) ok = mbar_wait(smem_u32(done), 0u, abort_flag, P.flag);
    __syncwarp();
    tc_fence_after();
    const int row = m0 + warp * 32 + lane;
    KahanF fro;
    if (EPI == EPI_UPDATE && P.c_tma) {
        // C tile -> the stage buffers (free once `done` has fired) by TMA, in 64-column chunks
        // that all start at once; D = C - alpha * acc in place in shared memory, each chunk
        // TMA-stored as soon as it is done.  Rows / columns outside the matrix are zero-filled
        // on load, clipped on store and left out of the sum of squares.
        ok = __syncthreads_and(ok) != 0;
        const int nch = (P.BN + CW - 1) / CW;
        float *sc = (float *)sbase;
        if (ok && threadIdx.x == 0) {
            for (int c = 0; c < nch; c++) {
                const uint32_t cb = smem_u32(&cbar[c]);
                mbar_expect_tx(cb, (uint32_t)(BM * CW * 4));
                tma_load_2d(base + (uint32_t)(c * BM * CW * 4), &maps.c, cb, m0, n0 + c * CW);
            }
        }
        const int r = warp * 32 + lane;
        for (int c = 0; ok && c < nch; c++) {
            const bool got = mbar_wait(smem_u32(&cbar[c]), 0u, abort_flag, P.flag);
            if (!__syncthreads_and(got)) break;
            float *tile = sc + (size_t)c * BM * CW;
#pragma unroll 1
            for (int cc = 0; cc < CW; cc += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * CW + cc), v);
#pragma unroll
                for (int t = 0; t < 16; t++) {
                    float *e = tile + (size_t)(cc + t) * BM + r;
                    const float nv = *e - P.alpha * v[t];
                    *e = nv;
                    const int col = n0 + c * CW + cc + t;
                    if (row < P.M && col < P.N) {
                        fro.add(nv * nv);
                        if (P.Shi) {
                            // the next products' operands, written while the value is in hand
                            const float h = __uint_as_float((__float_as_uint(nv) + 0x1000u) & 0xFFFFE000u);
                            P.Shi[(long long)row + (long long)col * P.lds] = h;
                            P.Slo[(long long)row + (long long)col * P.lds] = nv - h;
                            const __nv_bfloat16 bh = __float2bfloat16_rn(nv);
                            P.Bhi[(long long)row + (long long)col * P.ldb] = bh;
                            P.Blo[(long long)row + (long long)col * P.ldb] = __float2bfloat16_rn(nv - __bfloat162float(bh));
                        }
                    }
                }
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            if (threadIdx.x == 0) {
                tma_store_2d(&maps.d, base + (uint32_t)(c * BM * CW * 4), m0, n0 + c * CW);
                asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            }
        }
        if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    } else if (ok && EPI == EPI_UPDATE) {
        // C may alias D: each 16-column group of C is loaded into registers before any of
        // that group's stores, and the next group's loads are issued before this group is
        // stored, so a thread keeps 16 loads in flight instead of one
        const bool rv = row < P.M;
        const bool want_fro = P.fro_part != nullptr;
        float cnext[16];
        auto load_c = [&](int c0, float (&cv)[16]) {
#pragma unroll
            for (int t = 0; t < 16; t++) {
                const int col = n0 + c0 + t;
                cv[t] = (rv && col < P.N) ? P.C[(long long)row + (long long)col * P.ldc] : 0.f;
            }
        };
        load_c(0, cnext);
        for (int c0 = 0; c0 < P.BN; c0 += 16) {
            float cv[16], v[16];
#pragma unroll
            for (int t = 0; t < 16; t++) cv[t] = cnext[t];
            if (nkb > 0) tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            else {
#pragma unroll
                for (int t = 0; t < 16; t++) v[t] = 0.f;
            }
            if (c0 + 16 < P.BN) load_c(c0 + 16, cnext);
            if (rv) {
#pragma unroll
                for (int t = 0; t < 16; t++) {
                    const int col = n0 + c0 + t;
                    if (col < P.N) {
                        const float nv = cv[t] - P.alpha * v[t];
                        P.D[(long long)row + (long long)col * P.ldd] = nv;
                        if (want_fro) fro.add(nv * nv);
                    }
                }
            }
        }
    } else if (ok) {
        for (int c0 = 0; c0 < P.BN; c0 += 16) {
            float v[16];
            if (nkb > 0) tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            else {
#pragma unroll
                for (int t = 0; t < 16; t++) v[t] = 0.f;
            }
            if (row < P.M) {
#pragma unroll
                for (int t = 0; t < 16; t++) {
                    const int col = n0 + c0 + t;
                    if (col >= P.N) break;
                    if (EPI == EPI_STORE) {
                        P.D[(long long)row + (long long)col * P.ldd] = P.alpha * v[t];
                    } else if (EPI == EPI_PARTIAL) {
                        P.D[(long long)blockIdx.z * P.part_stride + (long long)row + (long long)col * P.ldd] = v[t];
                    } else {
                        const float nv = P.C[(long long)row + (long long)col * P.ldc] - P.alpha * v[t];
                        P.D[(long long)row + (long long)col * P.ldd] = nv;
                        fro.add(nv * nv);
                    }
                }
            }
        }
    }
    if (EPI == EPI_UPDATE && P.fro_part) {
        __shared__ double red[32];
        const double tot = block_sum(fro.value(), red);
        if (threadIdx.x == 0) P.fro_part[blockIdx.x + (long long)gridDim.x * blockIdx.y] = tot;
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 2) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
    }
}

// D = alpha * (sum of the split-K partial slabs).  The slabs are summed in FP32 with
// Neumaier's compensation (error ~2^-24 of the sum plus a second-order term), not in FP64:
// FP64 adds and conversions, one of each per slab and element, made this pass FP64-bound
// on GB300 (~1 TB/s).  Each thread reduces four consecutive rows of one column with 16-byte
// loads, four slabs per step (the slabs' leading dimension ldp and stride are multiples of
// 4 floats; rows M..ldp-1 are read and dropped).
struct Neumaier {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float t = s + x;
        c += (fabsf(s) >= fabsf(x)) ? ((s - t) + x) : ((x - t) + s);
        s = t;
    }
};
__global__ void splitk_reduce_kernel(const float *part, long long stride, int splits, int M, int N, long long ldp,
                                     float *D, long long ldd, float alpha) {
    const long long mq = ((long long)M + 3) / 4, total = mq * N, s4 = stride / 4;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long j = e / mq, i = (e - j * mq) * 4;
        const float4 *p = (const float4 *)(part + i + j * ldp);
        Neumaier a0, a1, a2, a3;
        int z = 0;
        for (; z + 4 <= splits; z += 4) {
            float4 v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) v[u] = __ldcs(p + (long long)(z + u) * s4);
#pragma unroll
            for (int u = 0; u < 4; u++) { a0.add(v[u].x); a1.add(v[u].y); a2.add(v[u].z); a3.add(v[u].w); }
        }
        for (; z < splits; z++) {
            const float4 v = __ldcs(p + (long long)z * s4);
            a0.add(v.x); a1.add(v.y); a2.add(v.z); a3.add(v.w);
        }
        float *d = D + i + j * ldd;
        d[0] = alpha * (a0.s + a0.c);
        if (i + 1 < M) d[1] = alpha * (a1.s + a1.c);
        if (i + 2 < M) d[2] = alpha * (a2.s + a2.c);
        if (i + 3 < M) d[3] = alpha * (a3.s + a3.c);
    }
}

// First pass for small outputs with many slabs: slab g*G <- sum of slabs g*G .. g*G+G-1
// (compensated), in place (group g reads and writes only its own slabs).
__global__ void splitk_group_kernel(float *part, long long stride, int splits, int G, int M, int N, long long ldp) {
    const long long mq = ((long long)M + 3) / 4, per = mq * N, s4 = stride / 4;
    const int ng = (splits + G - 1) / G;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < per * ng;
         e += (long long)gridDim.x * blockDim.x) {
        const long long g = e / per, r = e - g * per;
        const long long j = r / mq, i = (r - j * mq) * 4;
        float4 *p = (float4 *)(part + i + j * ldp);
        Neumaier a0, a1, a2, a3;
        const int z0 = (int)g * G, z1 = min(splits, z0 + G);
        for (int z = z0; z < z1; z++) {
            const float4 v = __ldcs(p + (long long)z * s4);
            a0.add(v.x); a1.add(v.y); a2.add(v.z); a3.add(v.w);
        }
        p[(long long)z0 * s4] = make_float4(a0.s + a0.c, a1.s + a1.c, a2.s + a2.c, a3.s + a3.c);
    }
}

static void splitk_reduce(cudaStream_t s, float *part, long long stride, int splits, int M, int N, long long ldp,
                          float *D, long long ldd, float alpha, int sms) {
    const long long total = ((long long)M + 3) / 4 * N;
    if (splits >= 16 && total < (long long)sms * 512) {
        // too few outputs to spread over the GPU: sum groups of 8 slabs in parallel first
        constexpr int G = 8;
        const long long work = total * ((splits + G - 1) / G);
        const unsigned g1 = (unsigned)std::max<long long>(1, std::min<long long>((work + 255) / 256, (long long)sms * 16));
        splitk_group_kernel<<<g1, 256, 0, s>>>(part, stride, splits, G, M, N, ldp);
        RSVD_LAUNCH_CK();
        stride *= G;
        splits = (splits + G - 1) / G;
    }
    const unsigned g = (unsigned)std::max<long long>(1, std::min<long long>((total + 255) / 256, (long long)sms * 16));
    splitk_reduce_kernel<<<g, 256, 0, s>>>(part, stride, splits, M, N, ldp, D, ldd, alpha);
    RSVD_LAUNCH_CK();
}

// ------------------------------------------------------------------ host side
using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                              const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeFn encode_fn() {
    static std::once_flag once;
    static EncodeFn fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeFn)p;
    });
    if (!fn) fail(RSVD_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    return fn;
}

// 2-D tensor map over a column-major-ish buffer: dim0 contiguous (extent e0), dim1 with
// stride (bytes); box {b0, b1}; 128B swizzle; out-of-bounds elements read as zero.
static CUtensorMap make_map(const void *ptr, int esz, long long e0, long long e1, long long stride_bytes, int b0,
                            int b1) {
    if (((uintptr_t)ptr & 15) || (stride_bytes & 15)) fail(RSVD_ERR_ARGUMENT, "tensor map: 16-byte alignment");
    if (b0 * esz > 128 || b1 > 256 || b0 <= 0 || b1 <= 0) fail(RSVD_ERR_ARGUMENT, "tensor map: bad box");
    CUtensorMap m;
    std::memset(&m, 0, sizeof m);
    cuuint64_t dims[2] = {(cuuint64_t)e0, (cuuint64_t)e1};
    cuuint64_t strides[1] = {(cuuint64_t)stride_bytes};
    cuuint32_t box[2] = {(cuuint32_t)b0, (cuuint32_t)b1};
    cuuint32_t es[2] = {1, 1};
    CUresult r = encode_fn()(&m, esz == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                             const_cast<void *>(ptr), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                             CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) fail(RSVD_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    return m;
}

// Unswizzled FP32 map for the update epilogue's C / D tiles: dim0 = rows (contiguous), box
// {BM, CW} (512-byte rows of the box, packed column after column in shared memory).
static CUtensorMap make_map_tile(const void *ptr, long long e0, long long e1, long long stride_bytes) {
    if (((uintptr_t)ptr & 15) || (stride_bytes & 15)) fail(RSVD_ERR_ARGUMENT, "tensor map: 16-byte alignment");
    CUtensorMap m;
    std::memset(&m, 0, sizeof m);
    cuuint64_t dims[2] = {(cuuint64_t)e0, (cuuint64_t)e1};
    cuuint64_t strides[1] = {(cuuint64_t)stride_bytes};
    cuuint32_t box[2] = {(cuuint32_t)BM, (cuuint32_t)CW};
    cuuint32_t es[2] = {1, 1};
    CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(ptr), dims, strides, box, es,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) fail(RSVD_ERR_CUDA, "cuTensorMapEncodeTiled failed (C/D tile)");
    return m;
}

// Raise a kernel's dynamic shared-memory limit on the current device to what the device's
// opt-in per-block maximum (227 KB on GB300) leaves after the kernel's static shared memory
// (the update epilogue's reduction scratch).
template <typename Kern>
static void set_max_dynamic_smem(Kern k, int dev) {
    cudaFuncAttributes fa{};
    RSVD_CK(cudaFuncGetAttributes(&fa, k));
    int optin = 0;
    RSVD_CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    RSVD_CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
}

template <int KIND, bool A_MN, int EPI>
static void launch(cudaStream_t s, dim3 grid, size_t smem, const Maps &maps, const Params &P) {
    auto k = tc_gemm_kernel<KIND, A_MN, EPI>;
    // function attributes are per device: set once per (instantiation, device)
    static std::atomic<bool> attr_set[128];
    const int dev = ctx().device;
    if (dev < 0 || dev >= 128) fail(RSVD_ERR_NO_DEVICE, "device ordinal out of range");
    if (!attr_set[dev].load(std::memory_order_acquire)) {
        set_max_dynamic_smem(k, dev);
        attr_set[dev].store(true, std::memory_order_release);
    }
    k<<<grid, NTHR, smem, s>>>(maps, P);
    RSVD_LAUNCH_CK();
    ctx().launches++;
    ctx().timing.gemm_launches++;
}

}  // namespace tc

// Public launchers (declared in rsvd_internal.h).
void tc_gemm_segs(cudaStream_t s, int kind, bool a_mn, int nseg, const TcSeg *seg, int M, int N, float alpha,
                  float *D, long long ldd, int epi, const float *C, long long ldc, double *fro_part, int splits_hint,
                  const TcSplitOut *so) {
    using namespace tc;
    const int esz = (kind == KIND_TF32) ? 4 : 2;
    const int KE = KB / esz;
    if (nseg < 1 || nseg > MAX_SEG) fail(RSVD_ERR_ARGUMENT, "tc_gemm: 1 to 3 K segments");
    if (M <= 0 || N <= 0) fail(RSVD_ERR_ARGUMENT, "tc_gemm: empty");
    int num_kb = 0, Ktot = 0;
    for (int g = 0; g < nseg; g++) {
        if (seg[g].K <= 0) fail(RSVD_ERR_ARGUMENT, "tc_gemm: empty K segment");
        num_kb += (seg[g].K + KE - 1) / KE;
        Ktot += seg[g].K;
    }
    // kind::tf32 with an MN-major A operand produced wrong products on GB300; only the
    // K-major form is used with tf32 (MN-major operands go through kind::f16 / bf16).
    if (kind == KIND_TF32 && a_mn) fail(RSVD_ERR_ARGUMENT, "tc_gemm: tf32 needs a K-major A operand");
    // column tiling: one CTA covers up to 512 columns as one MMA chunk (<= 256 columns) or
    // two EQUAL chunks (both use the same TMA box, so each box fills exactly its half of
    // the stage buffer); wider products tile N by 256.
    const int Npad16 = (N + 15) / 16 * 16;
    int BN, c0, c1;
    if (Npad16 <= 256) { BN = Npad16; c0 = BN; c1 = 0; }
    else if (N <= MAX_BN) { BN = (N + 31) / 32 * 32; c0 = c1 = BN / 2; }
    else { BN = 256; c0 = 256; c1 = 0; }
    const int ntiles = (N + BN - 1) / BN;
    const int mtiles = (M + BM - 1) / BM;
    // split-K so that the grid fills the GPU when row tiles are few
    int splits = 1;
    const int sms = std::max(1, ctx().sms);
    if (epi == EPI_STORE && splits_hint != 1) {
        // time model in units of one k-block of one CTA (one CTA per SM; a k-block moves
        // (BM + BN) x 128 bytes through shared memory at ~80 GB/s per SM on GB300):
        //   waves(z) x ceil(num_kb / z)  +  the split-K reduce, which writes and reads z
        //   FP32 partial slabs of M x N at ~6 TB/s.
        const int tiles = mtiles * ntiles;
        const double t_kb = (double)(BM + BN) * KB / 80e9;
        auto cost = [&](int z) {
            const double waves = (double)((tiles * z + sms - 1) / sms);
            const double main = waves * (double)((num_kb + z - 1) / z);
            const double red = (z > 1) ? (double)z * 8.0 * (double)M * (double)N / 6e12 / t_kb : 0.0;
            return main + red;
        };
        double best = cost(1);
        for (int z = 2; z <= 8; z++) {
            if (num_kb / z < 4) break;
            const double c = cost(z);
            if (c < best * 0.97) { best = c; splits = z; }
        }
        if (splits_hint > 1) splits = splits_hint;
    }
    const int kb_per_split = (num_kb + splits - 1) / splits;
    splits = (num_kb + kb_per_split - 1) / kb_per_split;

    const size_t stage_bytes = (size_t)A_BYTES + (size_t)BN * KB;
    int stages = (int)std::min<size_t>(8, (220 * 1024) / stage_bytes);
    if (stages < 2) fail(RSVD_ERR_ARGUMENT, "tc_gemm: tile does not fit in shared memory");
    const size_t smem = (size_t)stages * stage_bytes + 1024 + 64 + 16 * stages;

    // tensor maps: A either MN-major (dim0 = M) or K-major (dim0 = K); X K-major (dim0 = K)
    Maps maps;
    std::memset(&maps, 0, sizeof maps);
    Params P{};
    for (int g = 0; g < nseg; g++) {
        const TcSeg &q = seg[g];
        maps.a[g] = a_mn ? make_map(q.A, esz, M, q.K, q.lda * esz, KE, KE) : make_map(q.A, esz, q.K, M, q.lda * esz, KE, BM);
        maps.b[g] = make_map(q.X, esz, q.K, N, q.ldx * esz, KE, c0);
        P.seg_kb[g] = (q.K + KE - 1) / KE;
    }
    P.nseg = nseg;
    P.M = M; P.N = N; P.K = Ktot; P.BN = BN; P.chunk_n0 = c0; P.chunk_n1 = c1;
    P.num_kb = num_kb; P.kb_per_split = kb_per_split; P.stages = stages; P.alpha = alpha;
    P.flag = ctx().d_flags + FLAG_TIMEOUT;
    P.fro_part = fro_part;
    P.C = C; P.ldc = ldc;
    dim3 grid(mtiles, ntiles, splits);
    if (epi == EPI_UPDATE) {
        P.D = D; P.ldd = ldd;
        // C through shared memory by TMA when the tile fits in the stage buffers, the
        // 64-column chunks stay inside this CTA's columns, and M is a multiple of 4 (the
        // bulk store clipped a ragged row extent only at 16-byte granularity on GB300: with
        // M = 257 it wrote rows 257..259)
        const int nch = (BN + CW - 1) / CW;
        P.c_tma = M % 4 == 0 && BN <= 256 && (ntiles == 1 || BN % CW == 0) &&
                  (size_t)nch * BM * CW * 4 <= (size_t)stages * stage_bytes &&
                  ((uintptr_t)C % 16 == 0) && ((uintptr_t)D % 16 == 0) && (ldc * 4) % 16 == 0 && (ldd * 4) % 16 == 0;
        if (P.c_tma) {
            maps.c = make_map_tile(C, M, N, ldc * 4);
            maps.d = make_map_tile(D, M, N, ldd * 4);
            if (so) {
                P.Shi = so->hi; P.Slo = so->lo; P.lds = so->ld;
                P.Bhi = so->bhi; P.Blo = so->blo; P.ldb = so->ldb;
            }
        }
        if (kind == KIND_TF32) {
            if (a_mn) launch<KIND_TF32, true, EPI_UPDATE>(s, grid, smem, maps, P);
            else launch<KIND_TF32, false, EPI_UPDATE>(s, grid, smem, maps, P);
        } else {
            if (a_mn) launch<KIND_BF16, true, EPI_UPDATE>(s, grid, smem, maps, P);
            else launch<KIND_BF16, false, EPI_UPDATE>(s, grid, smem, maps, P);
        }
        if (so && !P.c_tma) {
            // the register epilogue does not write the splits: separate passes
            split_tf32(s, D, ldd, M, N, so->hi, so->lo, so->ld);
            split_bf16(s, DM<float>{D, M, N, ldd}, DM<__nv_bfloat16>{so->bhi, M, N, so->ldb},
                       DM<__nv_bfloat16>{so->blo, M, N, so->ldb});
        }
        return;
    }
    if (splits == 1) {
        P.D = D; P.ldd = ldd;
        if (kind == KIND_TF32) {
            if (a_mn) launch<KIND_TF32, true, EPI_STORE>(s, grid, smem, maps, P);
            else launch<KIND_TF32, false, EPI_STORE>(s, grid, smem, maps, P);
        } else {
            if (a_mn) launch<KIND_BF16, true, EPI_STORE>(s, grid, smem, maps, P);
            else launch<KIND_BF16, false, EPI_STORE>(s, grid, smem, maps, P);
        }
        return;
    }
    const long long ldp = ((long long)M + 31) / 32 * 32;
    const long long stride = ldp * N;
    DBuf part(sizeof(float) * (size_t)stride * splits, s);
    P.D = (float *)part.get(); P.ldd = ldp; P.part_stride = stride;
    if (kind == KIND_TF32) {
        if (a_mn) launch<KIND_TF32, true, EPI_PARTIAL>(s, grid, smem, maps, P);
        else launch<KIND_TF32, false, EPI_PARTIAL>(s, grid, smem, maps, P);
    } else {
        if (a_mn) launch<KIND_BF16, true, EPI_PARTIAL>(s, grid, smem, maps, P);
        else launch<KIND_BF16, false, EPI_PARTIAL>(s, grid, smem, maps, P);
    }
    splitk_reduce(s, (float *)part.get(), stride, splits, M, N, ldp, D, ldd, alpha, sms);
    ctx().launches++;
}

void tc_gemm(cudaStream_t s, int kind, bool a_mn, const void *A, long long lda, const void *X, long long ldx,
             int M, int N, int K, float alpha, float *D, long long ldd, int epi, const float *C, long long ldc,
             double *fro_part, int splits_hint) {
    if (K <= 0) fail(RSVD_ERR_ARGUMENT, "tc_gemm: empty");
    const TcSeg g{A, lda, X, ldx, K};
    tc_gemm_segs(s, kind, a_mn, 1, &g, M, N, alpha, D, ldd, epi, C, ldc, fro_part, splits_hint, nullptr);
}

// =====================================================================================
// Allocation-free variant of the split-K sketch product Y = A^T X (kind::tf32).
//
// For callers that cannot allocate GPU memory at the point of the call: code running
// under an external memory manager or budget that forbids driver allocations, callers
// that must not trigger the implicit synchronisation of cudaMalloc / cudaFree, and hosts
// that reserve all device memory up front.  Every other entry point of this library
// allocates stream-ordered workspace (and its first call creates a per-thread context);
// this one uses only the caller's buffers, the caller's stream, and a file-scope scratch
// array that every GPU that loads the library holds until process exit:
//   bytes [0, 256)   : device status word (bounded-wait timeout flag), cleared every call
//   bytes [256, ...) : split-K partial slabs (fully written before they are read)
// Limit: 2 slabs of round_up(n, 32) x w floats must fit in the scratch (32 MiB), i.e.
// round_up(n, 32) * w <= 4,194,272; larger products are rejected with RSVD_ERR_ARGUMENT.
// Set-up (once per device, on the first call made while that device is current) looks
// up the scratch array's device address with cudaGetSymbolAddress and sets the kernel's
// shared-memory limit; make that first call before any stream capture.  All calls share
// the one array, so calls that overlap on the GPU (other streams, other host threads on
// the same device) race on it: serialise them.
// =====================================================================================
namespace {
constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)32 << 20;
constexpr size_t NOALLOC_HEADER = 256;
}  // namespace

static __device__ __align__(256) unsigned char rsvd_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

namespace {
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[128] = {nullptr};

// Per-device set-up: the scratch array's device address and the kernel attribute.
void *noalloc_setup(int dev) {
    if (dev < 0 || dev >= 128) fail(RSVD_ERR_NO_DEVICE, "device ordinal out of range");
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (g_noalloc_ptr[dev]) return g_noalloc_ptr[dev];
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, rsvd_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        fail(RSVD_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch) failed: ") + cudaGetErrorString(e));
    }
    tc::set_max_dynamic_smem(tc::tc_gemm_kernel<tc::KIND_TF32, false, tc::EPI_PARTIAL>, dev);
    g_noalloc_ptr[dev] = p;
    return p;
}
}  // namespace

}  // namespace rsvd

extern "C" int rsvdpack_dev_sketch_t_noalloc(const float *dA, long long lda, int m, int n, const float *dX,
                                             long long ldx, int w, float *dY, long long ldy, void *stream) {
    using namespace rsvd;
    using namespace rsvd::tc;
    try {
        rsvdpack_clear_error();
        cudaStream_t s = (cudaStream_t)stream;
        if (!dA || !dX || !dY) fail(RSVD_ERR_ARGUMENT, "null device pointer");
        if (m <= 0 || n <= 0 || w <= 0) fail(RSVD_ERR_ARGUMENT, "empty product");
        if (lda < m || ldx < m || ldy < n) fail(RSVD_ERR_ARGUMENT, "bad leading dimension");
        // the call ends by waiting for its stream, which a capturing stream cannot do
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        RSVD_CK(cudaStreamIsCapturing(s, &cap));
        if (cap != cudaStreamCaptureStatusNone) fail(RSVD_ERR_ARGUMENT, "the stream is capturing (this call is synchronous)");
        int dev = -1;
        RSVD_CK(cudaGetDevice(&dev));
        int major = 0, minor = 0, sms = 0;
        RSVD_CK(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
        RSVD_CK(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
        RSVD_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        if (!(major == 10 && minor == 3)) fail(RSVD_ERR_NO_DEVICE, "needs an sm_103 (GB300) device");
        unsigned char *scratch = (unsigned char *)noalloc_setup(dev);

        // Y (n x w) = A^T X : M = n, N = w, K = m, A is the K-major operand
        const int M = n, N = w, K = m;
        const int KE = KB / 4;
        const int Npad16 = (N + 15) / 16 * 16;
        int BN, c0, c1;
        if (Npad16 <= 256) { BN = Npad16; c0 = BN; c1 = 0; }
        else if (N <= MAX_BN) { BN = (N + 31) / 32 * 32; c0 = c1 = BN / 2; }
        else { BN = 256; c0 = 256; c1 = 0; }
        const int ntiles = (N + BN - 1) / BN, mtiles = (M + BM - 1) / BM;
        const int num_kb = (K + KE - 1) / KE;
        const long long ldp = ((long long)M + 31) / 32 * 32;
        const long long stride = ldp * N;
        const long long max_slabs = (long long)((NOALLOC_SCRATCH_BYTES - NOALLOC_HEADER) / (sizeof(float) * (size_t)stride));
        if (max_slabs < 2)
            fail(RSVD_ERR_ARGUMENT, "product too large for the no-allocation scratch: need round_up(n,32)*w <= 4194272");
        if (num_kb < 2) fail(RSVD_ERR_ARGUMENT, "m too small to split (needs m > 32)");
        int splits = 2;
        const int tiles = mtiles * ntiles;
        for (int z = 2; z <= 8 && z <= max_slabs && z <= num_kb; z++)
            if ((long long)tiles * z <= (long long)sms) splits = z;
        const int kb_per_split = (num_kb + splits - 1) / splits;
        splits = (num_kb + kb_per_split - 1) / kb_per_split;

        const size_t stage_bytes = (size_t)A_BYTES + (size_t)BN * KB;
        const int stages = (int)std::min<size_t>(8, (220 * 1024) / stage_bytes);
        const size_t smem = (size_t)stages * stage_bytes + 1024 + 64 + 16 * stages;
        Maps maps;
        std::memset(&maps, 0, sizeof maps);
        maps.a[0] = make_map(dA, 4, K, M, lda * 4, KE, BM);
        maps.b[0] = make_map(dX, 4, K, N, ldx * 4, KE, c0);
        int *flag = (int *)scratch;
        float *part = (float *)(scratch + NOALLOC_HEADER);
        Params P{};
        P.M = M; P.N = N; P.K = K; P.BN = BN; P.chunk_n0 = c0; P.chunk_n1 = c1;
        P.num_kb = num_kb; P.kb_per_split = kb_per_split; P.stages = stages; P.alpha = 1.0f;
        P.nseg = 1; P.seg_kb[0] = num_kb;
        P.flag = flag; P.D = part; P.ldd = ldp; P.part_stride = stride;
        RSVD_CK(cudaMemsetAsync(flag, 0, sizeof(int), s));
        tc_gemm_kernel<KIND_TF32, false, EPI_PARTIAL><<<dim3(mtiles, ntiles, splits), NTHR, smem, s>>>(maps, P);
        RSVD_LAUNCH_CK();
        splitk_reduce(s, part, stride, splits, M, N, ldp, dY, ldy, 1.0f, sms);
        int h = 0;
        RSVD_CK(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
        RSVD_CK(cudaStreamSynchronize(s));
        if (h) fail(RSVD_ERR_TIMEOUT, "a bounded device-side wait gave up");
        return RSVD_OK;
    } catch (const Error &e) {
        set_error(e.code, std::string("rsvdpack_dev_sketch_t_noalloc: ") + e.what());
        return e.code;
    }
}

namespace rsvd {

// ---------------------------------------------------------------- 3xTF32 products
// FP32-accurate products on the tf32 tensor pipe: x = hi + lo with hi = x rounded to TF32
// (10 mantissa bits, representable exactly, so the MMA's operand conversion leaves it
// unchanged) and lo = x - hi (exact in FP32); A^T X = hi_A^T hi_X + lo_A^T hi_X + hi_A^T lo_X,
// the dropped lo_A^T lo_X term and the TF32 rounding of lo being ~2^-22 relative.
namespace {
__global__ void split_tf32_kernel(const float *X, long long ldx, long long r, long long c, float *hi, float *lo,
                                  long long ldo) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < r * c;
         e += (long long)gridDim.x * blockDim.x) {
        const long long j = e / r, i = e - j * r;
        const float x = X[i + j * ldx];
        const float h = __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
        hi[i + j * ldo] = h;
        lo[i + j * ldo] = x - h;
    }
}
}  // namespace

namespace {
__global__ void add_kernel(float *D, long long ldd, const float *T, long long ldt, int M, int N) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)M * N;
         e += (long long)gridDim.x * blockDim.x) {
        const long long j = e / M, i = e - j * M;
        D[i + j * ldd] += T[i + j * ldt];
    }
}
}  // namespace

void split_tf32(cudaStream_t s, const float *X, long long ldx, long long r, long long c, float *hi, float *lo,
                long long ldo) {
    if (r * c == 0) return;
    const long long want = (r * c + 255) / 256, cap = (long long)std::max(1, ctx().sms) * 16;
    split_tf32_kernel<<<(unsigned)std::min(want, cap), 256, 0, s>>>(X, ldx, r, c, hi, lo, ldo);
    RSVD_LAUNCH_CK();
    ctx().launches++;
}

// D (M x N) = A^T X with A K-major (K x M, lda) and X (K x N, ldx), both given split.
// The tensor core's FP32 accumulation truncates at every MMA step, so its error grows with
// the number of steps in one accumulation chain, not with sqrt(K): a 2048-long chain of
// the dominant hi x hi product already costs ~1e-5 relative.  That product is therefore
// split along K into chains of ~256 (FP32 in TMEM within a chain, compensated FP32 across chains,
// ~1e-6 relative), its partial slabs capped at 1 GiB.  The two correction terms, 2^-11
// smaller, are one two-segment product with chains of ~2048 into a temporary that one
// elementwise pass adds.
void tc_gemm_3xtf32(cudaStream_t s, const float *Ahi, const float *Alo, long long lda, const float *Xhi,
                    const float *Xlo, long long ldx, int M, int N, int K, float *D, long long ldd) {
    const long long ldt = ((long long)M + 31) / 32 * 32;
    const long long slab_cap = std::max(1ll, (1ll << 30) / (ldt * N * (long long)sizeof(float)));
    const int splits_hh = (int)std::max(1ll, std::min({(K + 255) / 256ll, slab_cap, 128ll}));
    // corrections: chains of ~1024 where the output has many tiles; where it has few (a Gram,
    // M = N = l), enough splits to fill two waves of the GPU, up to the hi x hi split count
    const long long tiles = ((long long)M + 127) / 128 * (N <= 512 ? 1 : ((long long)N + 255) / 256);
    const long long fill = (2ll * std::max(1, ctx().sms) + tiles - 1) / tiles;
    const int splits = (int)std::max<long long>(1, std::max<long long>(std::min(32, K / 1024),
                                                                        std::min<long long>(splits_hh, fill)));
    DBuf t(sizeof(float) * (size_t)ldt * N, s);
    tc_gemm(s, tc::KIND_TF32, false, Ahi, lda, Xhi, ldx, M, N, K, 1.0f, D, ldd, tc::EPI_STORE, nullptr, 0, nullptr,
            splits_hh);
    const TcSeg corr[2] = {{Alo, lda, Xhi, ldx, K}, {Ahi, lda, Xlo, ldx, K}};
    tc_gemm_segs(s, tc::KIND_TF32, false, 2, corr, M, N, 1.0f, (float *)t.get(), ldt, tc::EPI_STORE, nullptr, 0,
                 nullptr, splits);
    const long long want = ((long long)M * N + 255) / 256, cap = (long long)std::max(1, ctx().sms) * 16;
    add_kernel<<<(unsigned)std::min(want, cap), 256, 0, s>>>(D, ldd, (const float *)t.get(), ldt, M, N);
    RSVD_LAUNCH_CK();
    ctx().launches++;
}

// C (M x N) -= A^T X from split operands, the three terms as one three-segment update
// (lo x hi, hi x lo, then hi x hi: the small terms accumulate first).  fro_part: per-CTA
// sums of squares of the new C (tc_gemm's update layout), or null.
void tc_update_3xtf32(cudaStream_t s, const float *Ahi, const float *Alo, long long lda, const float *Xhi,
                      const float *Xlo, long long ldx, int M, int N, int K, float *Cm, long long ldc,
                      double *fro_part, const TcSplitOut *so) {
    const TcSeg g[3] = {{Alo, lda, Xhi, ldx, K}, {Ahi, lda, Xlo, ldx, K}, {Ahi, lda, Xhi, ldx, K}};
    tc_gemm_segs(s, tc::KIND_TF32, false, 3, g, M, N, 1.0f, Cm, ldc, tc::EPI_UPDATE, Cm, ldc, fro_part, 1, so);
}

}  // namespace rsvd
