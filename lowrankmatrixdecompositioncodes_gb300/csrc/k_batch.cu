// k_batch.cu -- batched fixed-rank rSVD: many independent FP32 matrices of uneven size in one
// persistent launch (the reference has one matrix per call; low_rank_svd_rand_decomp_fixed_rank,
// rank_revealing_algorithms_intel_mkl.c:73-174, is applied to every matrix of the batch with
// vnum = 1).
//
// Each CTA pops matrices from a device work queue and runs the whole pipeline on one matrix:
//   Om (n x l)   Philox4x32-10 Gaussians, drawn straight into shared memory (never in HBM)
//   Y = A Om     A streamed in 64 x 32 tiles
//   [q-1 power rounds: Yo = cqr(Y); Z = A^T Yo; Zo = cqr(Z); Y = A Zo]
//   Q = cqr2(Y) ; Bt = A^T Q ; (Qh, Rh) = cqr2(Bt) ; Rh = Uh S Vh^T (Jacobi in shared memory)
//   U = Q Vh(:, 1:k) ; V = Qh Uh(:, 1:k)
// cqr = CholeskyQR (Gram, Cholesky and triangular inverse in shared memory), all FP32.
// Tall intermediates live in a per-CTA slab of global memory (L2-resident across the CTA's
// work).  Matrices are taken largest-first (the host sorts the queue) to balance the tail.
#include "k_batch.h"

#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

namespace rsvd {

// Shared memory and slab sizes for a batch whose largest matrix is (mmax x nmax), l <= lmax.
size_t batch_smem_bytes(int nmax, int lmax) {
    const size_t phase1 = (size_t)nmax * lmax + 3 + 32 * ATP;
    const size_t L2 = (size_t)lmax * lmax;
    const size_t small = 4 * L2 + 33 * 96 + 2 * L2 + 96 + 32 * 96 + 3 + 32 * ATP + 64;
    return sizeof(float) * std::max(phase1, small) + 64;
}

// A configuration of the batched kernel: lanes per Jacobi pair and the column-group offset of
// the register-tiled products.
struct BatchCfg {
    int lp = 8, cuadd = 0;
};

void batch_rsvd_launch(cudaStream_t s, const BatchItem *d_items, int count, int *d_queue, float *d_work, long long slab,
                       long long ldw, unsigned long long seed, int q, int s_, int *d_flag, int nctas, size_t smem,
                       BatchCfg cfg) {
    switch (cfg.lp) {
        case 4: batch_rsvd_launch_lp4(s, d_items, count, d_queue, d_work, slab, ldw, seed, q, s_, d_flag, nctas, smem, cfg.cuadd); break;
        case 16: batch_rsvd_launch_lp16(s, d_items, count, d_queue, d_work, slab, ldw, seed, q, s_, d_flag, nctas, smem, cfg.cuadd); break;
        case 32: batch_rsvd_launch_lp32(s, d_items, count, d_queue, d_work, slab, ldw, seed, q, s_, d_flag, nctas, smem, cfg.cuadd); break;
        default: batch_rsvd_launch_lp8(s, d_items, count, d_queue, d_work, slab, ldw, seed, q, s_, d_flag, nctas, smem, cfg.cuadd); break;
    }
}

// ---------------------------------------------------------------- the autotuner
// The candidates (lanes per Jacobi pair x column-group offset) are timed on a strided sample of
// the sorted batch (every count / S-th matrix, S = min(count, 2 x SMs), so that the sample has
// the batch's size mix) with CUDA events, one warm-up and two timed launches each, and the fastest
// is used.  Choices are kept per batch class -- (max k + p, max n / 64, max m / 64, q) -- in a
// table that lives for the process and in a text file (RSVDPACK_TUNE_FILE, else
// $HOME/.cache/rsvdpack/batch_tune.txt; one "key lp cuadd ms" line per class), read at the first
// plan of a class and appended to after each new tuning.
struct TuneEntry {
    BatchCfg cfg;
    double ms = 0.0;
};
std::mutex g_tune_mu;
std::map<std::string, TuneEntry> g_tune;
bool g_tune_loaded = false;

std::string tune_path() {
    if (const char *p = std::getenv("RSVDPACK_TUNE_FILE")) return p;
    const char *h = std::getenv("HOME");
    return std::string(h ? h : ".") + "/.cache/rsvdpack/batch_tune.txt";
}

void tune_load_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    std::FILE *f = std::fopen(tune_path().c_str(), "r");
    if (!f) return;
    char key[128];
    int lp, cu;
    double ms;
    while (std::fscanf(f, "%127s %d %d %lf", key, &lp, &cu, &ms) == 4) {
        if ((lp == 4 || lp == 8 || lp == 16 || lp == 32) && (cu == 0 || cu == 1)) {
            TuneEntry e;
            e.cfg.lp = lp;
            e.cfg.cuadd = cu;
            e.ms = ms;
            g_tune[key] = e;
        }
    }
    std::fclose(f);
}

void tune_store_locked(const std::string &key, const TuneEntry &e) {
    g_tune[key] = e;
    const std::string path = tune_path();
    const size_t slash = path.find_last_of('/');
    if (slash != std::string::npos) {
        // create the directory chain (best effort: an unwritable location only loses persistence)
        std::string dir;
        for (size_t i = 0; i <= slash; i++) {
            dir += path[i];
            if (path[i] == '/' && i > 0) mkdir(dir.c_str(), 0755);
        }
    }
    if (std::FILE *f = std::fopen(path.c_str(), "a")) {
        std::fprintf(f, "%s %d %d %.6f\n", key.c_str(), e.cfg.lp, e.cfg.cuadd, e.ms);
        std::fclose(f);
    }
}

}  // namespace rsvd

// ============================================================ plan API (extern "C")
struct rsvdpack_batch_plan {
    int count = 0;
    int lp = 8, cuadd = 0, tuned = 0;   // chosen configuration; tuned: 1 measured now, 2 from the table
    double tune_ms = 0.0;               // the chosen configuration's time on the tuning sample
    rsvd::DBuf items, queue, work, flag;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t stream = nullptr;
};

extern "C" {

rsvdpack_batch_plan *rsvdpack_batch_plan_create(int count, const int *m, const int *n, const int *k, int p, int q,
                                                int s, const float *const *dA, const long long *lda,
                                                float *const *dU, const long long *ldu, double *const *dS,
                                                float *const *dV, const long long *ldv, unsigned long long seed) {
    using namespace rsvd;
    rsvdpack_batch_plan *plan = nullptr;
    try {
        rsvdpack_clear_error();
        if (count <= 0 || !m || !n || !k || !dA || !lda || !dU || !ldu || !dS || !dV || !ldv)
            fail(RSVD_ERR_ARGUMENT, "null or empty batch description");
        if (p < 0 || (q >= 2 && s < 1)) fail(RSVD_ERR_ARGUMENT, "need p >= 0 and s >= 1");
        Ctx &cx = ctx();
        std::vector<BatchItem> items((size_t)count);
        int mmax = 1, nmax = 1, lmax = 1;
        for (int i = 0; i < count; i++) {
            const int l = k[i] + p;
            if (m[i] <= 0 || n[i] <= 0 || k[i] < 1 || l > std::min(m[i], n[i]))
                fail(RSVD_ERR_ARGUMENT, "batch item " + std::to_string(i) + ": need 1 <= k, k + p <= min(m, n)");
            if (l > 72) fail(RSVD_ERR_ARGUMENT, "batch item " + std::to_string(i) + ": k + p above 72");
            if (lda[i] < m[i] || ldu[i] < m[i] || ldv[i] < n[i]) fail(RSVD_ERR_ARGUMENT, "bad leading dimension");
            items[(size_t)i] = BatchItem{dA[i], lda[i], dU[i], ldu[i], dS[i], dV[i], ldv[i], m[i], n[i], k[i], l, i, 0};
            mmax = std::max(mmax, m[i]);
            nmax = std::max(nmax, n[i]);
            lmax = std::max(lmax, l);
        }
        const size_t smem = batch_smem_bytes(nmax, lmax);
        if (smem > 220 * 1024) fail(RSVD_ERR_ARGUMENT, "batch: n * (k + p) too large for shared memory (n <= 760 at k+p = 72)");
        // largest problems first: the queue hands them out early, small ones fill the tail
        std::stable_sort(items.begin(), items.end(), [](const BatchItem &a, const BatchItem &b) {
            return (long long)a.m * a.n * a.l > (long long)b.m * b.n * b.l;
        });
        plan = new rsvdpack_batch_plan();
        plan->count = count;
        plan->stream = cx.stream;
        cudaStream_t st = cx.stream;
        plan->items = DBuf(sizeof(BatchItem) * (size_t)count, st);
        RSVD_CK(cudaMemcpyAsync(plan->items.get(), items.data(), sizeof(BatchItem) * (size_t)count,
                                cudaMemcpyHostToDevice, st));
        const int nctas = std::max(1, std::min(cx.sms, count));
        const long long ldw = pad_ld(std::max(mmax, nmax));
        const long long slab = 2 * ldw * 96;
        plan->work = DBuf(sizeof(float) * (size_t)slab * nctas, st);
        plan->queue = DBuf(sizeof(int), st);
        plan->flag = DBuf(sizeof(int), st);
        RSVD_CK(cudaStreamSynchronize(st));
        // ---- configuration: the table entry of this batch class, else tuned on a sample
        BatchCfg cfg;
        {
            char keyb[128];
            std::snprintf(keyb, sizeof keyb, "l%d_n%d_m%d_q%d", lmax, (nmax + 63) / 64, (mmax + 63) / 64, q);
            const std::string key = keyb;
            std::lock_guard<std::mutex> g(g_tune_mu);
            tune_load_locked();
            auto it = g_tune.find(key);
            if (it != g_tune.end()) {
                cfg = it->second.cfg;
                plan->tune_ms = it->second.ms;
                plan->tuned = 2;
            } else if (!std::getenv("RSVDPACK_NO_TUNE")) {
                const int S = std::min(count, 2 * std::max(1, cx.sms));
                std::vector<BatchItem> sample((size_t)S);
                for (int i = 0; i < S; i++) sample[(size_t)i] = items[(size_t)((long long)i * count / S)];
                DBuf sitems(sizeof(BatchItem) * (size_t)S, st);
                RSVD_CK(cudaMemcpyAsync(sitems.get(), sample.data(), sizeof(BatchItem) * (size_t)S,
                                        cudaMemcpyHostToDevice, st));
                cudaEvent_t e0, e1;
                RSVD_CK(cudaEventCreate(&e0));
                RSVD_CK(cudaEventCreate(&e1));
                double best = 1e300;
                const int snct = std::max(1, std::min(cx.sms, S));
                for (int lp : {4, 8, 16, 32})
                    for (int cu : {0, 1}) {
                        BatchCfg c;
                        c.lp = lp;
                        c.cuadd = cu;
                        float tot = 0.f;
                        for (int rep = 0; rep < 3; rep++) {
                            RSVD_CK(cudaMemsetAsync(plan->queue.get(), 0, sizeof(int), st));
                            RSVD_CK(cudaMemsetAsync(plan->flag.get(), 0, sizeof(int), st));
                            RSVD_CK(cudaEventRecord(e0, st));
                            batch_rsvd_launch(st, (const BatchItem *)sitems.get(), S, (int *)plan->queue.get(),
                                              (float *)plan->work.get(), slab, ldw, seed, q, s,
                                              (int *)plan->flag.get(), snct, smem, c);
                            RSVD_CK(cudaEventRecord(e1, st));
                            RSVD_CK(cudaEventSynchronize(e1));
                            float ms = 0.f;
                            RSVD_CK(cudaEventElapsedTime(&ms, e0, e1));
                            if (rep > 0) tot += ms;
                        }
                        const double ms = tot / 2.0;
                        if (ms < best) {
                            best = ms;
                            cfg = c;
                        }
                    }
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                TuneEntry e;
                e.cfg = cfg;
                e.ms = best;
                tune_store_locked(key, e);
                plan->tune_ms = best;
                plan->tuned = 1;
            }
        }
        plan->lp = cfg.lp;
        plan->cuadd = cfg.cuadd;
        // one persistent launch (plus the two counter resets) captured in a CUDA graph
        RSVD_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        cudaMemsetAsync(plan->queue.get(), 0, sizeof(int), st);
        cudaMemsetAsync(plan->flag.get(), 0, sizeof(int), st);
        batch_rsvd_launch(st, (const BatchItem *)plan->items.get(), count, (int *)plan->queue.get(),
                          (float *)plan->work.get(), slab, ldw, seed, q, s, (int *)plan->flag.get(), nctas, smem, cfg);
        RSVD_CK(cudaStreamEndCapture(st, &plan->graph));
        RSVD_CK(cudaGraphInstantiate(&plan->exec, plan->graph, 0));
        return plan;
    } catch (const Error &e) {
        set_error(e.code, std::string("rsvdpack_batch_plan_create: ") + e.what());
        if (plan) {
            cudaStreamEndCapture(plan->stream, &plan->graph);
            delete plan;
        }
        return nullptr;
    }
}

int rsvdpack_batch_plan_execute(rsvdpack_batch_plan *plan) {
    using namespace rsvd;
    try {
        rsvdpack_clear_error();
        if (!plan || !plan->exec) fail(RSVD_ERR_ARGUMENT, "null plan");
        RSVD_CK(cudaGraphLaunch(plan->exec, plan->stream));
        int bad = 0;
        RSVD_CK(cudaMemcpyAsync(&bad, plan->flag.get(), sizeof(int), cudaMemcpyDeviceToHost, plan->stream));
        RSVD_CK(cudaStreamSynchronize(plan->stream));
        if (bad) fail(RSVD_ERR_NUMERIC, std::to_string(bad) + " batch item(s) broke down in CholeskyQR");
        return RSVD_OK;
    } catch (const Error &e) {
        set_error(e.code, std::string("rsvdpack_batch_plan_execute: ") + e.what());
        return e.code;
    }
}

int rsvdpack_batch_plan_info(const rsvdpack_batch_plan *plan, int *lanes_per_pair, int *col_group_offset,
                             int *tuned, double *tune_ms) {
    if (!plan) return RSVD_ERR_ARGUMENT;
    if (lanes_per_pair) *lanes_per_pair = plan->lp;
    if (col_group_offset) *col_group_offset = plan->cuadd;
    if (tuned) *tuned = plan->tuned;
    if (tune_ms) *tune_ms = plan->tune_ms;
    return RSVD_OK;
}

void rsvdpack_batch_plan_destroy(rsvdpack_batch_plan *plan) {
    if (!plan) return;
    if (plan->exec) cudaGraphExecDestroy(plan->exec);
    if (plan->graph) cudaGraphDestroy(plan->graph);
    delete plan;
}

}  // extern "C"
