// api.cu -- extern "C" drop-in for RSVDPACK's C API (include/rsvdpack.h, Part 1).
//
// Each entry point: validate -> upload A (host double, column-major) to the device in the
// engine's working precision -> run the device algorithm (engine.cu) -> allocate the
// outputs with matrix_new / vector_new and copy them back.  Errors never exit(): the
// outputs are set to NULL and rsvdpack_last_error() reports the cause.
#include "engine.h"
#include "k_common.cuh"

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <utility>
#include <vector>

#include <sys/mman.h>

using namespace rsvd;

// Host element type of the library being compiled: double, or float in the oneAPI-variant one.
using real = rsvd_real;

namespace rsvd {
// Default precision mode of this library's reference API (read once by the option setup):
// FP64 for the double-data libraries (the reference's arithmetic), FP32 for the float-data one.
int api_default_precision() {
#ifdef RSVDPACK_REAL32
    return RSVD_PREC_FP32;
#else
    return RSVD_PREC_FP64;
#endif
}
}  // namespace rsvd

namespace {

using Clock = std::chrono::steady_clock;
double ms_since(Clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

template <typename F>
void guarded(const char *fn, F &&body) {
    try {
        rsvdpack_clear_error();
        body();
    } catch (const Error &e) {
        set_error(e.code, std::string(fn) + ": " + e.what());
    } catch (const std::bad_alloc &) {
        set_error(RSVD_ERR_ALLOC, std::string(fn) + ": host allocation failed");
    } catch (const std::exception &e) {
        set_error(RSVD_ERR_CUDA, std::string(fn) + ": " + e.what());
    }
}

void need(bool ok, const char *what) {
    if (!ok) fail(RSVD_ERR_ARGUMENT, what);
}

// The engine's dimensions are int (offsets and element counts are 64-bit throughout), so the
// 64-bit-index library takes any matrix whose rows and columns each fit an int: m * n may
// exceed 2^31.
void check_mat(const mat *M) {
    need(M != nullptr && M->d != nullptr, "null matrix");
    need(M->nrows > 0 && M->ncols > 0, "empty matrix");
    need((long long)M->nrows <= INT_MAX && (long long)M->ncols <= INT_MAX, "dimension above 2^31 - 1");
}

// Rank, oversampling, power and step arguments of the 64-bit-index library: each must fit an int.
template <typename... Ts>
void need_int(Ts... v) {
    need(((v >= (rsvd_int)INT_MIN && v <= (rsvd_int)INT_MAX) && ...), "argument outside the int range");
}

// Working precision of the tall products for this call.
bool use_fp32_path() {
    const int p = ctx().opts.precision;
    return p != RSVD_PREC_FP64 && p != RSVD_PREC_FP64X;
}

template <typename T>
DMat<T> upload(const mat *M) {
    cudaStream_t s = ctx().stream;
    const i64 m = M->nrows, n = M->ncols;
    if (ctx().pageable_access) {
        // the conversion kernel reads the caller's (pageable) host matrix over NVLink-C2C:
        // one pass at the link's bandwidth, no staging copy and no device temporary.  In the
        // tensor-core modes a large A also gets its BF16 copy (the MN-major products read it) in
        // the same pass, where the extra device writes hide under the link-bound read.
        DMat<T> A(m, n, s, false);
        const int prec = ctx().opts.precision;
        if constexpr (std::is_same<T, float>::value) {
            if ((prec == RSVD_PREC_TF32 || prec == RSVD_PREC_BF16) && m * n >= (1ll << 22)) {
                DMat<__nv_bfloat16> Ab(m, n, s, false);
                convert_f32_bf16<real>(s, DM<real>{M->d, m, n, m}, A.v, Ab.v);
                RSVD_CK(cudaStreamSynchronize(s));
                adopt_bf16_copy(A.v, std::move(Ab));
                return A;
            }
        }
        convert<real, T>(s, DM<real>{M->d, m, n, m}, A.v);
        RSVD_CK(cudaStreamSynchronize(s));     // the caller may reuse M->d on return
        return A;
    }
    if (std::is_same<T, real>::value) {
        DMat<T> A(m, n, s, false);
        RSVD_CK(cudaMemcpy2DAsync(A.v.p, sizeof(T) * A.v.ld, M->d, sizeof(real) * m, sizeof(real) * m, n,
                                  cudaMemcpyHostToDevice, s));
        return A;
    }
    DMat<real> tmp(m, n, s, false);
    RSVD_CK(cudaMemcpy2DAsync(tmp.v.p, sizeof(real) * tmp.v.ld, M->d, sizeof(real) * m, sizeof(real) * m, n,
                              cudaMemcpyHostToDevice, s));
    DMat<T> A(m, n, s, false);
    convert<real, T>(s, tmp.v, A.v);
    RSVD_CK(cudaStreamSynchronize(s));
    return A;
}

// An output matrix the engine overwrites entirely: same ownership as matrix_new (freed
// with matrix_delete / free), but for large sizes 2 MB aligned with a transparent-huge-page
// hint and not zeroed, so that filling it costs a few page faults instead of one per 4 KB.
mat *matrix_new_output(rsvd_int nrows, rsvd_int ncols) {
    const size_t bytes = sizeof(real) * (size_t)std::max<rsvd_int>(nrows, 0) * (size_t)std::max<rsvd_int>(ncols, 0);
    if (bytes < ((size_t)4 << 20)) return matrix_new(nrows, ncols);
    mat *M = (mat *)std::malloc(sizeof(mat));
    if (!M) return nullptr;
    void *p = nullptr;
    const size_t align = (size_t)2 << 20;
    if (posix_memalign(&p, align, (bytes + align - 1) / align * align) != 0) {
        std::free(M);
        return nullptr;
    }
    madvise(p, (bytes + align - 1) / align * align, MADV_HUGEPAGE);
    M->nrows = nrows;
    M->ncols = ncols;
    M->d = (real *)p;
    return M;
}

// Host reductions over whole matrices: a fixed split into REDUCE_CHUNKS contiguous chunks, each
// summed in double by one of up to 16 threads, the chunk sums then added in chunk order -- the
// result does not depend on the thread count.  f(i) returns the (num, den) terms of element i.
constexpr int REDUCE_CHUNKS = 64;
template <typename F>
std::pair<double, double> host_reduce(size_t n, F f) {
    std::vector<double> num(REDUCE_CHUNKS, 0.0), den(REDUCE_CHUNKS, 0.0);
    auto run = [&](int c) {
        const size_t a = n * (size_t)c / REDUCE_CHUNKS, b = n * (size_t)(c + 1) / REDUCE_CHUNKS;
        double x = 0.0, y = 0.0;
        for (size_t i = a; i < b; i++) {
            const auto t = f(i);
            x += t.first;
            y += t.second;
        }
        num[(size_t)c] = x;
        den[(size_t)c] = y;
    };
    const int nt = n < ((size_t)1 << 20) ? 1 : (int)std::min<unsigned>(16, std::max(1u, std::thread::hardware_concurrency()));
    if (nt == 1) {
        for (int c = 0; c < REDUCE_CHUNKS; c++) run(c);
    } else {
        std::vector<std::thread> th;
        for (int t = 0; t < nt; t++)
            th.emplace_back([&, t] {
                for (int c = t; c < REDUCE_CHUNKS; c += nt) run(c);
            });
        for (auto &x : th) x.join();
    }
    double x = 0.0, y = 0.0;
    for (int c = 0; c < REDUCE_CHUNKS; c++) {
        x += num[(size_t)c];
        y += den[(size_t)c];
    }
    return {x, y};
}

// Pinned host staging for device-to-host copies (per thread, grown on demand).
struct PinnedStage {
    void *p = nullptr;
    size_t n = 0;
    ~PinnedStage() {
        if (p) cudaFreeHost(p);
    }
    void *get(size_t bytes) {
        if (bytes > n) {
            if (p) RSVD_CK(cudaFreeHost(p));
            p = nullptr;
            n = 0;
            RSVD_CK(cudaHostAlloc(&p, bytes, cudaHostAllocDefault));
            n = bytes;
        }
        return p;
    }
};
thread_local PinnedStage t_stage;

// Host copy from the pinned stage into the (pageable) output, split over a few threads.
void parallel_copy(real *dst, const real *src, size_t count) {
    const size_t bytes = count * sizeof(real);
    const int nt = bytes < ((size_t)8 << 20) ? 1 : 8;
    if (nt == 1) {
        std::memcpy(dst, src, bytes);
        return;
    }
    std::vector<std::thread> th;
    const size_t per = (count + nt - 1) / nt;
    for (int t = 0; t < nt; t++) {
        const size_t a = std::min(count, (size_t)t * per), b = std::min(count, a + per);
        if (a < b) th.emplace_back([=] { std::memcpy(dst + a, src + a, (b - a) * sizeof(real)); });
    }
    for (auto &x : th) x.join();
}

template <typename T>
mat *download(DM<T> a) {
    cudaStream_t s = ctx().stream;
    mat *M = matrix_new_output((rsvd_int)a.r, (rsvd_int)a.c);
    if (!M) throw std::bad_alloc();
    if (a.r * a.c == 0) return M;
    const size_t count = (size_t)a.r * (size_t)a.c;
    real *stage = (real *)t_stage.get(sizeof(real) * count);
    if (std::is_same<T, real>::value) {
        RSVD_CK(cudaMemcpy2DAsync(stage, sizeof(real) * a.r, a.p, sizeof(T) * a.ld, sizeof(real) * a.r, a.c,
                                  cudaMemcpyDeviceToHost, s));
        RSVD_CK(cudaStreamSynchronize(s));
    } else {
        DMat<real> tmp(a.r, a.c, s, false);
        convert<T, real>(s, a, tmp.v);
        RSVD_CK(cudaMemcpy2DAsync(stage, sizeof(real) * a.r, tmp.v.p, sizeof(real) * tmp.v.ld,
                                  sizeof(real) * a.r, a.c, cudaMemcpyDeviceToHost, s));
        RSVD_CK(cudaStreamSynchronize(s));
    }
    parallel_copy(M->d, stage, count);
    return M;
}

// An output of known size, allocated and pre-faulted by a host thread while the device
// works, then filled by the device: with pageable access the conversion kernel writes FP64
// straight into the caller-visible host buffer (its pages already present, so no faults from
// the device side); otherwise through the pinned stage as in download().
struct OutputPrefetch {
    mat *M = nullptr;
    std::thread th;
    OutputPrefetch(i64 r, i64 c) {
        th = std::thread([this, r, c] {
            M = matrix_new_output(r, c);
            if (!M) return;
            volatile char *b = (volatile char *)M->d;
            const size_t bytes = sizeof(real) * (size_t)r * (size_t)c;
            for (size_t off = 0; off < bytes; off += 4096) b[off] = 0;
        });
    }
    ~OutputPrefetch() {
        if (th.joinable()) th.join();
        if (M) matrix_delete(M);                 // not taken: an exception unwound the call
    }
    template <typename T>
    mat *fill(DM<T> a) {
        th.join();
        if (!M) throw std::bad_alloc();
        mat *out = M;
        M = nullptr;
        cudaStream_t s = ctx().stream;
        if (a.r * a.c == 0) return out;
        if (ctx().pageable_access) {
            convert<T, real>(s, a, DM<real>{out->d, a.r, a.c, a.r});
            RSVD_CK(cudaStreamSynchronize(s));
            return out;
        }
        const size_t count = (size_t)a.r * (size_t)a.c;
        real *stage = (real *)t_stage.get(sizeof(real) * count);
        DMat<real> tmp;
        const real *src = (const real *)a.p;
        long long lds = a.ld;
        if (!std::is_same<T, real>::value) {
            tmp = DMat<real>(a.r, a.c, s, false);
            convert<T, real>(s, a, tmp.v);
            src = tmp.v.p;
            lds = tmp.v.ld;
        }
        RSVD_CK(cudaMemcpy2DAsync(stage, sizeof(real) * a.r, src, sizeof(real) * lds, sizeof(real) * a.r, a.c,
                                  cudaMemcpyDeviceToHost, s));
        RSVD_CK(cudaStreamSynchronize(s));
        parallel_copy(out->d, stage, count);
        return out;
    }
};

mat *diag_mat(const std::vector<double> &d) {
    const int k = (int)d.size();
    mat *S = matrix_new(k, k);
    for (int i = 0; i < k; i++) S->d[(size_t)i * k + i] = (real)d[(size_t)i];
    return S;
}

vec *index_vec(const std::vector<int> &I) {
    vec *v = vector_new((rsvd_int)I.size());
    for (size_t i = 0; i < I.size(); i++) v->d[i] = (real)I[i];
    return v;
}

void begin_call() {
    Ctx &c = ctx();
    c.opts = global_opts();
    std::memset(&c.timing, 0, sizeof c.timing);
    c.launches = 0;
    phase_reset();
}

// Device entry points read caller memory: order the engine stream (non-blocking) after
// all work already queued on the legacy default stream.
void order_after_default_stream() {
    thread_local cudaEvent_t ev = nullptr;
    if (!ev) RSVD_CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    RSVD_CK(cudaEventRecord(ev, 0));
    RSVD_CK(cudaStreamWaitEvent(ctx().stream, ev, 0));
}

void end_call(Clock::time_point t0) {
    Ctx &c = ctx();
    release_operand_cache();
    phase_collect();
    check_device_flags(c);
    c.timing.total_ms = ms_since(t0);
    c.timing.kernel_launches = c.launches;
}

template <typename T>
void svd_outputs(SvdOut<T> &r, mat **U, mat **S, mat **V) {
    *U = download<T>(r.U.v);
    *V = download<T>(r.V.v);
    *S = diag_mat(r.S);
}

template <typename T>
void run_fixed_rank(mat *M, int k, int p, int vnum, int q, int s, mat **U, mat **S, mat **V) {
    auto t0 = Clock::now();
    OutputPrefetch pu(M->nrows, k), pv(M->ncols, k);          // U: m x k, V: n x k
    DMat<T> A = upload<T>(M);
    ctx().timing.upload_ms = ms_since(t0);
    SvdOut<T> r = svd_fixed_rank<T>(A.v, k, p, vnum, q, s);
    auto t1 = Clock::now();
    *U = pu.fill<T>(r.U.v);
    *V = pv.fill<T>(r.V.v);
    *S = diag_mat(r.S);
    ctx().timing.download_ms = ms_since(t1);
    end_call(t0);
}

template <typename T>
void run_blockrand(mat *M, int k, int p, double TOL, int vnum, int kstep, int q, int s, rsvd_int *frank, mat **U,
                   mat **S, mat **V) {
    auto t0 = Clock::now();
    DMat<T> A = upload<T>(M);
    int f = 0;
    SvdOut<T> r = svd_blockrand<T>(A.v, k, p, TOL, vnum, kstep, q, s, &f);
    svd_outputs<T>(r, U, S, V);
    if (frank) *frank = f;
    end_call(t0);
}

template <typename T>
void run_qb(mat *M, int kstep, int nstep, double TOL, int q, int s, rsvd_int *frank, mat **Q, mat **B,
            QbRule rule = QB_PB_NEW) {
    auto t0 = Clock::now();
    DMat<T> A = upload<T>(M);
    QBOut<T> r = qb_blocked<T>(A.v, kstep, nstep, TOL, q, s, rule);
    *Q = download<T>(r.Q.v);
    *B = download<T>(r.B.v);
    if (frank) *frank = r.frank;
    end_call(t0);
}

}  // namespace

extern "C" {

// ============================================================ storage (MVF:8-63)
mat *matrix_new(rsvd_int nrows, rsvd_int ncols) {
    mat *M = (mat *)std::malloc(sizeof(mat));
    if (!M) return nullptr;
    M->nrows = nrows;
    M->ncols = ncols;
    const size_t n = (size_t)(nrows > 0 ? nrows : 0) * (size_t)(ncols > 0 ? ncols : 0);
    M->d = (real *)std::calloc(n ? n : 1, sizeof(real));
    return M;
}

vec *vector_new(rsvd_int nrows) {
    vec *v = (vec *)std::malloc(sizeof(vec));
    if (!v) return nullptr;
    v->nrows = nrows;
    v->d = (real *)std::calloc(nrows > 0 ? (size_t)nrows : 1, sizeof(real));
    return v;
}

void matrix_delete(mat *M) {
    if (!M) return;
    std::free(M->d);
    std::free(M);
}

void vector_delete(vec *v) {
    if (!v) return;
    std::free(v->d);
    std::free(v);
}

void matrix_set_element(mat *M, rsvd_int i, rsvd_int j, real val) { M->d[(size_t)j * M->nrows + i] = val; }
real matrix_get_element(mat *M, rsvd_int i, rsvd_int j) { return M->d[(size_t)j * M->nrows + i]; }
void vector_set_element(vec *v, rsvd_int i, real val) { v->d[i] = val; }
real vector_get_element(vec *v, rsvd_int i) { return v->d[i]; }

constexpr rsvd_int FILE_ROWS = 64;   // rows per block of the binary-file transposition

// m, n as rsvd_int (int32; int64 in the 64-bit-index and float libraries, as the reference's
// 64-bit and oneAPI variants write them), then m*n values of the element type in row-major order
// (MVF:77-133; oneapi_code/matrix_vector_functions_one_api.c:71-130)
mat *matrix_load_from_binary_file(char *fname) {
    FILE *fp = std::fopen(fname, "rb");
    if (!fp) {
        set_error(RSVD_ERR_ARGUMENT, std::string("cannot open ") + fname);
        return nullptr;
    }
    rsvd_int hdr[2] = {0, 0};
    if (std::fread(hdr, sizeof(rsvd_int), 2, fp) != 2 || hdr[0] <= 0 || hdr[1] <= 0) {
        std::fclose(fp);
        set_error(RSVD_ERR_ARGUMENT, "bad matrix file header");
        return nullptr;
    }
    const rsvd_int m = hdr[0], n = hdr[1];
    mat *M = matrix_new_output(m, n);     // every entry is written below
    if (!M) {
        std::fclose(fp);
        set_error(RSVD_ERR_ALLOC, "host allocation failed");
        return nullptr;
    }
    // FILE_ROWS rows at a time, transposed by FILE_ROWS x FILE_ROWS tiles into the column-major
    // matrix: every write is a contiguous run of a column
    std::vector<real> blk((size_t)FILE_ROWS * (size_t)n);
    for (rsvd_int i0 = 0; i0 < m; i0 += FILE_ROWS) {
        const rsvd_int nb = std::min<rsvd_int>(FILE_ROWS, m - i0);
        if (std::fread(blk.data(), sizeof(real), (size_t)nb * n, fp) != (size_t)nb * n) {
            std::fclose(fp);
            matrix_delete(M);
            set_error(RSVD_ERR_ARGUMENT, "truncated matrix file");
            return nullptr;
        }
        for (rsvd_int j0 = 0; j0 < n; j0 += FILE_ROWS)
            for (rsvd_int j = j0; j < std::min<rsvd_int>(n, j0 + FILE_ROWS); j++) {
                real *dst = M->d + (size_t)j * m + i0;
                const real *src = blk.data() + j;
                for (rsvd_int r = 0; r < nb; r++) dst[r] = src[(size_t)r * n];
            }
    }
    std::fclose(fp);
    return M;
}

void matrix_write_to_binary_file(mat *M, char *fname) {
    FILE *fp = std::fopen(fname, "wb");
    if (!fp) {
        set_error(RSVD_ERR_ARGUMENT, std::string("cannot open ") + fname);
        return;
    }
    const rsvd_int hdr[2] = {M->nrows, M->ncols};
    const rsvd_int m = M->nrows, n = M->ncols;
    std::fwrite(hdr, sizeof(rsvd_int), 2, fp);
    std::vector<real> blk((size_t)FILE_ROWS * (size_t)n);
    for (rsvd_int i0 = 0; i0 < m; i0 += FILE_ROWS) {
        const rsvd_int nb = std::min<rsvd_int>(FILE_ROWS, m - i0);
        for (rsvd_int j0 = 0; j0 < n; j0 += FILE_ROWS)
            for (rsvd_int j = j0; j < std::min<rsvd_int>(n, j0 + FILE_ROWS); j++) {
                const real *src = M->d + (size_t)j * m + i0;
                real *dst = blk.data() + j;
                for (rsvd_int r = 0; r < nb; r++) dst[(size_t)r * n] = src[r];
            }
        std::fwrite(blk.data(), sizeof(real), (size_t)nb * n, fp);
    }
    std::fclose(fp);
}

void matrix_copy(mat *D, mat *S) {
    std::memcpy(D->d, S->d, sizeof(real) * (size_t)S->nrows * (size_t)S->ncols);
}

// Mt = M^T by 64 x 64 tiles
void matrix_build_transpose(mat *Mt, mat *M) {
    const rsvd_int m = M->nrows, n = M->ncols, T = 64;
    for (rsvd_int j0 = 0; j0 < n; j0 += T)
        for (rsvd_int i0 = 0; i0 < m; i0 += T)
            for (rsvd_int i = i0; i < std::min<rsvd_int>(m, i0 + T); i++)
                for (rsvd_int j = j0; j < std::min<rsvd_int>(n, j0 + T); j++)
                    Mt->d[(size_t)i * Mt->nrows + j] = M->d[(size_t)j * m + i];
}

// host reductions accumulate in double for either element type
real get_matrix_frobenius_norm(mat *M) {
    const real *a = M->d;
    const auto r = host_reduce((size_t)M->nrows * (size_t)M->ncols, [a](size_t i) {
        const double v = (double)a[i];
        return std::pair<double, double>(v * v, 0.0);
    });
    return (real)std::sqrt(r.first);
}

real get_percent_error_between_two_mats(mat *A, mat *B) {
    const real *a = A->d, *b = B->d;
    const auto r = host_reduce((size_t)A->nrows * (size_t)A->ncols, [a, b](size_t i) {
        const double d = (double)a[i] - (double)b[i];
        return std::pair<double, double>(d * d, (double)a[i] * (double)a[i]);
    });
    return (real)(100.0 * std::sqrt(r.first) / std::sqrt(r.second));
}

// MVF:299-311
real vector_get2norm(vec *v) {
    double acc = 0.0;
    for (rsvd_int i = 0; i < v->nrows; i++) acc += (double)v->d[i] * (double)v->d[i];
    return (real)std::sqrt(acc);
}

// MVF:490-499: D(i,i) = data(i) for the rows of D; the rest of D is left as it is
void initialize_diagonal_matrix(mat *D, vec *data) {
    for (rsvd_int i = 0; i < D->nrows; i++) D->d[(size_t)i * D->nrows + i] = data->d[i];
}

// MVF:504-515: D = I (the reference writes D(i,i) for every row; here the diagonal stops at
// min(m, n), inside the matrix)
void initialize_identity_matrix(mat *D) {
    std::memset(D->d, 0, sizeof(real) * (size_t)D->nrows * (size_t)D->ncols);
    for (rsvd_int i = 0; i < std::min(D->nrows, D->ncols); i++) D->d[(size_t)i * D->nrows + i] = (real)1;
}

// MVF:582-604: column j of M to / from a vector of M->nrows entries
void matrix_get_col(mat *M, rsvd_int j, vec *column_vec) {
    std::memcpy(column_vec->d, M->d + (size_t)j * M->nrows, sizeof(real) * (size_t)M->nrows);
}
void matrix_set_col(mat *M, rsvd_int j, vec *column_vec) {
    std::memcpy(M->d + (size_t)j * M->nrows, column_vec->d, sizeof(real) * (size_t)M->nrows);
}

#include "mat_helpers.h"

#if defined(RSVDPACK_REAL32)
// oneapi_code/matrix_vector_functions_one_api.c:1511-1513
real get_seconds_frac(real start, real end) { return end - start; }
#else
double get_seconds_frac(struct timeval start_timeval, struct timeval end_timeval) {
    const long secs = end_timeval.tv_sec - start_timeval.tv_sec;
    const long micros = secs * 1000000 + end_timeval.tv_usec - start_timeval.tv_usec;
    return micros / 1e6;
}
#endif

void initialize_random_matrix(mat *M) {
    guarded("initialize_random_matrix", [&] {
        check_mat(M);
        begin_call();
        DMat<double> Om = make_omega<double>(M->nrows, M->ncols);
        mat *tmp = download<double>(Om.v);
        std::memcpy(M->d, tmp->d, sizeof(real) * (size_t)M->nrows * (size_t)M->ncols);
        matrix_delete(tmp);
    });
}

static void host_gemm(const char *fn, bool ta, bool tb, mat *A, mat *B, mat *C) {
    guarded(fn, [&] {
        check_mat(A); check_mat(B); check_mat(C);
        begin_call();
        DMat<double> dA = upload<double>(A), dB = upload<double>(B);
        DMat<double> dC(C->nrows, C->ncols, ctx().stream, false);
        gemm<double>(ctx().stream, ta, tb, 1.0, dA.v, dB.v, 0.0, dC.v);
        mat *r = download<double>(dC.v);
        std::memcpy(C->d, r->d, sizeof(real) * (size_t)C->nrows * (size_t)C->ncols);
        matrix_delete(r);
    });
}

void matrix_matrix_mult(mat *A, mat *B, mat *C) { host_gemm("matrix_matrix_mult", false, false, A, B, C); }
void matrix_transpose_matrix_mult(mat *A, mat *B, mat *C) { host_gemm("matrix_transpose_matrix_mult", true, false, A, B, C); }
void matrix_matrix_transpose_mult(mat *A, mat *B, mat *C) { host_gemm("matrix_matrix_transpose_mult", false, true, A, B, C); }

// y = M x, y = M^T x (MVF:565-580): the same FP64 GEMM with one column
void matrix_vector_mult(mat *M, vec *x, vec *y) {
    mat xm{x->nrows, 1, x->d}, ym{y->nrows, 1, y->d};
    host_gemm("matrix_vector_mult", false, false, M, &xm, &ym);
}
void matrix_transpose_vector_mult(mat *M, vec *x, vec *y) {
    mat xm{x->nrows, 1, x->d}, ym{y->nrows, 1, y->d};
    host_gemm("matrix_transpose_vector_mult", true, false, M, &xm, &ym);
}

// Minv = Minv^-1 for an upper-triangular Minv, in place (MVF:532-535, LAPACK dtrtri 'U' 'N': the
// upper triangle is overwritten, the strictly lower part is left as it is): the engine's FP64
// triangular solve against the identity
void invert_upper_triangular_matrix(mat *Minv) {
    guarded("invert_upper_triangular_matrix", [&] {
        check_mat(Minv);
        need(Minv->nrows == Minv->ncols, "matrix must be square");
        begin_call();
        auto t0 = Clock::now();
        cudaStream_t s = ctx().stream;
        const i64 n = Minv->nrows;
        DMat<double> R = upload<double>(Minv);
        DMat<double> I(n, n, s, false), X(n, n, s, false);
        set_identity(s, I.v);
        trsm_left_upper(s, R.v, I.v, X.v);
        mat *h = download<double>(X.v);
        for (i64 j = 0; j < n; j++)
            for (i64 i = 0; i <= j; i++) Minv->d[(size_t)j * n + i] = h->d[(size_t)j * n + i];
        matrix_delete(h);
        end_call(t0);
    });
}

// A X = B for an upper-triangular A (MVF:1477-1523).  solve_type 2 inverts A in place and
// multiplies, as the reference does; every other type (1: dtrsm; 3: the SVD pseudo-inverse, the
// same X for the nonsingular triangular A the routine is for; others: dtrsv per column) is the
// engine's FP64 triangular solve.  The order is B->nrows, as in the reference.
void upper_triangular_system_solve(mat *A, mat *B, mat *X, rsvd_int solve_type) {
    if (solve_type == 2) {
        invert_upper_triangular_matrix(A);
        if (rsvdpack_last_error() == RSVD_OK) matrix_matrix_mult(A, B, X);
        return;
    }
    guarded("upper_triangular_system_solve", [&] {
        check_mat(A);
        check_mat(B);
        check_mat(X);
        need(A->nrows >= B->nrows && A->ncols >= B->nrows, "A must hold a B->nrows x B->nrows triangle");
        need(X->nrows == B->nrows && X->ncols == B->ncols, "X must have B's shape");
        begin_call();
        auto t0 = Clock::now();
        cudaStream_t s = ctx().stream;
        DMat<double> dA = upload<double>(A), dB = upload<double>(B);
        DMat<double> dX(B->nrows, B->ncols, s, false);
        trsm_left_upper(s, dA.v.sub(0, 0, B->nrows, B->nrows), dB.v, dX.v);
        mat *h = download<double>(dX.v);
        std::memcpy(X->d, h->d, sizeof(real) * (size_t)X->nrows * (size_t)X->ncols);
        matrix_delete(h);
        end_call(t0);
    });
}

// Eigenvalues ascending into evals, eigenvectors into the columns of S (MVF:1206-1209, LAPACK dsyev
// 'V' 'U': the upper triangle of S defines the matrix).  The engine's FP64 one-sided Jacobi SVD of
// S + sigma I with sigma = ||S||_F, which is positive semidefinite, so that its singular pairs are
// eigenpairs: lambda = sv - sigma.  Absolute accuracy of every eigenvalue ~n eps ||S||_F (the
// Jacobi's backward error on the shifted matrix; dsyev's bound is of order eps ||S||_2), so
// eigenvalues far below ||S||_F carry correspondingly fewer correct digits.  A Jacobi run that hits its sweep limit
// returns RSVD_ERR_NUMERIC instead of unconverged pairs.
void compute_evals_and_evecs_of_symm_matrix(mat *S, vec *evals) {
    guarded("compute_evals_and_evecs_of_symm_matrix", [&] {
        check_mat(S);
        need(S->nrows == S->ncols, "matrix must be square");
        need(evals != nullptr && evals->d != nullptr && evals->nrows >= S->nrows, "evals shorter than S");
        begin_call();
        auto t0 = Clock::now();
        cudaStream_t s = ctx().stream;
        const i64 n = S->nrows;
        std::vector<double> g((size_t)n * (size_t)n);
        double fro2 = 0.0;
        for (i64 j = 0; j < n; j++)
            for (i64 i = 0; i <= j; i++) {
                const double v = (double)S->d[(size_t)j * n + i];
                g[(size_t)j * n + i] = g[(size_t)i * n + j] = v;
                fro2 += (i == j ? 1.0 : 2.0) * v * v;
            }
        const double sigma = fro2 > 0.0 ? std::sqrt(fro2) : 1.0;
        for (i64 i = 0; i < n; i++) g[(size_t)i * n + i] += sigma;
        DMat<double> G(n, n, s, false), U(n, n, s, false), V(n, n, s, false);
        DBuf svb(sizeof(double) * (size_t)n, s);
        RSVD_CK(cudaMemcpy2DAsync(G.v.p, sizeof(double) * G.v.ld, g.data(), sizeof(double) * n, sizeof(double) * n, n,
                                  cudaMemcpyHostToDevice, s));
        jacobi_small<double>(s, G.v, U.v, V.v, (double *)svb.get(), ctx().d_flags + FLAG_JACOBI_NOCONV, false);
        std::vector<double> sv((size_t)n);
        RSVD_CK(cudaMemcpyAsync(sv.data(), svb.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, s));
        mat *hv = download<double>(V.v);                 // synchronises the stream
        int noconv = 0;
        RSVD_CK(cudaMemcpyAsync(&noconv, ctx().d_flags + FLAG_JACOBI_NOCONV, sizeof(int), cudaMemcpyDeviceToHost, s));
        RSVD_CK(cudaStreamSynchronize(s));
        if (noconv) {
            matrix_delete(hv);
            fail(RSVD_ERR_NUMERIC, "Jacobi iteration did not converge");
        }
        for (i64 j = 0; j < n; j++) {                    // the SVD is descending; eigenvalues ascending
            const i64 src = n - 1 - j;
            evals->d[j] = (real)(sv[(size_t)src] - sigma);
            std::memcpy(S->d + (size_t)j * n, hv->d + (size_t)src * n, sizeof(real) * (size_t)n);
        }
        matrix_delete(hv);
        end_call(t0);
    });
}

// A X = B by LU with partial pivoting (MVF:1525-1531, LAPACK dgesv): X and B receive the solution;
// A is left as it is (the reference leaves its LU factors there)
void square_matrix_system_solve(mat *A, mat *X, mat *B) {
    guarded("square_matrix_system_solve", [&] {
        check_mat(A);
        check_mat(B);
        check_mat(X);
        need(A->nrows == A->ncols && B->nrows == A->nrows, "need a square A and B with A's rows");
        need(X->nrows == B->nrows && X->ncols == B->ncols, "X must have B's shape");
        begin_call();
        auto t0 = Clock::now();
        DMat<double> dA = upload<double>(A), dB = upload<double>(B);
        if (!lu_solve(ctx().stream, dA.v, dB.v, ctx().d_flags + FLAG_NONFINITE))
            fail(RSVD_ERR_NUMERIC, "singular matrix");
        mat *h = download<double>(dB.v);
        const size_t cnt = (size_t)X->nrows * (size_t)X->ncols;
        std::memcpy(X->d, h->d, sizeof(real) * cnt);
        std::memcpy(B->d, h->d, sizeof(real) * cnt);
        matrix_delete(h);
        end_call(t0);
    });
}

// P = U S V^T (MVF:1304-1318)
void form_svd_product_matrix(mat *U, mat *S, mat *V, mat *P) {
    mat *SVt = matrix_new(S->nrows, V->nrows);
    matrix_matrix_transpose_mult(S, V, SVt);
    matrix_matrix_mult(U, SVt, P);
    matrix_delete(SVt);
}

// P = C U R (MVF:1322-1336)
void form_cur_product_matrix(mat *C, mat *U, mat *R, mat *P) {
    mat *CU = matrix_new(C->nrows, U->ncols);
    matrix_matrix_mult(C, U, CU);
    matrix_matrix_mult(CU, R, P);
    matrix_delete(CU);
}

// ============================================================ decompositions
void low_rank_svd_rand_decomp_fixed_rank(mat *M, rsvd_int k, rsvd_int p, rsvd_int vnum, rsvd_int q, rsvd_int s, rsvd_int *frank, mat **U,
                                         mat **S, mat **V) {
    (void)frank;   // not written by the reference (RRA:73-234)
    *U = *S = *V = nullptr;
    guarded("low_rank_svd_rand_decomp_fixed_rank", [&] {
        check_mat(M);
        need_int(k, p, vnum, q, s);
        need(k >= 1 && p >= 0, "need k >= 1 and p >= 0");
        need(k + p <= std::min(M->nrows, M->ncols), "k + p exceeds min(m, n)");
        need(q < 2 || s >= 1, "s must be >= 1 when q >= 2");
        begin_call();
        if (use_fp32_path()) run_fixed_rank<float>(M, k, p, vnum, q, s, U, S, V);
        else run_fixed_rank<double>(M, k, p, vnum, q, s, U, S, V);
    });
}

void low_rank_svd_blockrand_decomp_fixed_rank_or_prec(mat *M, rsvd_int k, rsvd_int p, real TOL, rsvd_int vnum, rsvd_int kstep, rsvd_int q,
                                                      rsvd_int s, rsvd_int *frank, mat **U, mat **S, mat **V) {
    *U = *S = *V = nullptr;
    guarded("low_rank_svd_blockrand_decomp_fixed_rank_or_prec", [&] {
        check_mat(M);
        need_int(k, p, vnum, kstep, q, s);
        need(kstep >= 1 && p >= 0, "need kstep >= 1 and p >= 0");
        need(q < 1 || s >= 1, "s must be >= 1");
        begin_call();
        if (use_fp32_path()) run_blockrand<float>(M, k, p, TOL, vnum, kstep, q, s, frank, U, S, V);
        else run_blockrand<double>(M, k, p, TOL, vnum, kstep, q, s, frank, U, S, V);
    });
}

static void qb_pb_new(const char *fn, mat *M, rsvd_int kstep, rsvd_int nstep, real TOL, rsvd_int q, rsvd_int s,
                      rsvd_int *frank, mat **Q, mat **B) {
    *Q = *B = nullptr;
    guarded(fn, [&] {
        check_mat(M);
        need_int(kstep, nstep, q, s);
        need(kstep >= 1, "need kstep >= 1");
        need(q < 1 || s >= 1, "s must be >= 1");
        need((long long)kstep * nstep <= (long long)std::min(M->nrows, M->ncols) || kstep > std::min(M->nrows, M->ncols) / 2,
             "kstep * nstep exceeds min(m, n)");
        begin_call();
        if (use_fp32_path()) run_qb<float>(M, kstep, nstep, TOL, q, s, frank, Q, B);
        else run_qb<double>(M, kstep, nstep, TOL, q, s, frank, Q, B);
    });
}

void randQB_pb_new(mat *M, rsvd_int kstep, rsvd_int nstep, real TOL, rsvd_int q, rsvd_int s, rsvd_int *frank, mat **Q,
                   mat **B) {
    qb_pb_new("randQB_pb_new", M, kstep, nstep, TOL, q, s, frank, Q, B);
}

// oneapi_code/rank_revealing_algorithms_one_api.c:605-815: the randQB_pb_new algorithm
void randQB_pb2(mat *M, rsvd_int kstep, rsvd_int nstep, real TOL, rsvd_int q, rsvd_int s, rsvd_int *frank, mat **Q,
                mat **B) {
    qb_pb_new("randQB_pb2", M, kstep, nstep, TOL, q, s, frank, Q, B);
}

// RRA:1425-1570 (one_api.c:451-600): nstep blocks, no TOL mode, no kstep rule, every block
// after the first re-orthogonalised
void randQB_pb(mat *M, rsvd_int kstep, rsvd_int nstep, rsvd_int q, rsvd_int s, mat **Q, mat **B) {
    *Q = *B = nullptr;
    guarded("randQB_pb", [&] {
        check_mat(M);
        need_int(kstep, nstep, q, s);
        need(kstep >= 1 && nstep >= 1, "need kstep >= 1 and nstep >= 1");
        need(q < 1 || s >= 1, "s must be >= 1");
        need((long long)kstep * nstep <= (long long)std::min(M->nrows, M->ncols), "kstep * nstep exceeds min(m, n)");
        begin_call();
        if (use_fp32_path()) run_qb<float>(M, kstep, nstep, 0.0, q, s, nullptr, Q, B, QB_PB);
        else run_qb<double>(M, kstep, nstep, 0.0, q, s, nullptr, Q, B, QB_PB);
    });
}

// MVF:1214-1263: Householder QR with LAPACK's reflectors (FP64 on the device); Q m x n, and R
// n x n whose upper triangle is written
static void host_qr(const char *fn, mat *M, mat *Q, mat *R) {
    guarded(fn, [&] {
        check_mat(M);
        need(Q != nullptr && Q->d != nullptr, "null Q");
        need(M->nrows >= M->ncols, "QR needs rows >= columns");
        need(Q->nrows == M->nrows && Q->ncols == M->ncols, "Q must be m x n");
        if (R) need(R->d != nullptr && R->nrows == M->ncols && R->ncols == M->ncols, "R must be n x n");
        begin_call();
        auto t0 = Clock::now();
        DMat<double> W = upload<double>(M);
        const i64 n = M->ncols;
        DMat<double> dQ(M->nrows, n, ctx().stream, false), dR(n, n, ctx().stream, true);
        householder_qr<double>(ctx().stream, W.v, dQ.v, dR.v);
        mat *hq = download<double>(dQ.v);
        std::memcpy(Q->d, hq->d, sizeof(real) * (size_t)M->nrows * (size_t)n);
        matrix_delete(hq);
        if (R) {
            mat *hr = download<double>(dR.v);
            for (i64 j = 0; j < n; j++)
                for (i64 i = 0; i <= j; i++) R->d[(size_t)j * n + i] = hr->d[(size_t)j * n + i];
            matrix_delete(hr);
        }
        end_call(t0);
    });
}

void compact_QR_factorization(mat *M, mat *Q, mat *R) { host_qr("compact_QR_factorization", M, Q, R); }
void QR_factorization_getQ(mat *M, mat *Q) { host_qr("QR_factorization_getQ", M, Q, nullptr); }

void pivotedQR_mkl(mat *M, mat **Q, mat **R, vec **I) {
    *Q = *R = nullptr;
    *I = nullptr;
    guarded("pivotedQR_mkl", [&] {
        check_mat(M);
        begin_call();
        auto t0 = Clock::now();
        DMat<double> A = upload<double>(M);
        PivQROut r = pivoted_qr_full(A.v);
        *Q = download<double>(r.Q.v);
        *R = download<double>(r.R.v);
        *I = index_vec(r.I);
        end_call(t0);
    });
}

void pivoted_QR_of_specified_rank_or_prec(mat *M, rsvd_int k, real TOL, rsvd_int *frank, mat **Qk, mat **Rk, vec **I) {
    *Qk = *Rk = nullptr;
    *I = nullptr;
    guarded("pivoted_QR_of_specified_rank_or_prec", [&] {
        check_mat(M);
        need_int(k);
        need(k <= std::min(M->nrows, M->ncols), "k exceeds min(m, n)");
        begin_call();
        auto t0 = Clock::now();
        DMat<double> A = upload<double>(M);
        PivQROut r = pivoted_qr_partial(A.v, k, TOL);
        *Qk = download<double>(r.Q.v);
        *Rk = download<double>(r.R.v);
        *I = index_vec(r.I);
        if (frank) *frank = r.frank;
        end_call(t0);
    });
}

void pivoted_QR_of_specified_rank(mat *M, rsvd_int k, rsvd_int *frank, mat **Qk, mat **Rk, vec **I) {
    *Qk = *Rk = nullptr;
    *I = nullptr;
    guarded("pivoted_QR_of_specified_rank", [&] {
        check_mat(M);
        need_int(k);
        need(k >= 1 && k <= std::min(M->nrows, M->ncols), "need 1 <= k <= min(m, n)");
        begin_call();
        auto t0 = Clock::now();
        DMat<double> A = upload<double>(M);
        PivQROut r = pivoted_qr_partial(A.v, k, 0.0, 0.0);
        *Qk = download<double>(r.Q.v);
        *Rk = download<double>(r.R.v);
        *I = index_vec(r.I);
        if (frank) *frank = r.frank;
        end_call(t0);
    });
}

void id_decomp_fixed_rank_or_prec(mat *M, rsvd_int k, real TOL, rsvd_int *frank, vec **I, mat **T) {
    *I = nullptr;
    *T = nullptr;
    guarded("id_decomp_fixed_rank_or_prec", [&] {
        check_mat(M);
        need_int(k);
        need(k <= std::min(M->nrows, M->ncols), "k exceeds min(m, n)");
        begin_call();
        auto t0 = Clock::now();
        DMat<double> A = upload<double>(M);
        IdOut r = id_det(A.v, k, TOL);
        *I = index_vec(r.I);
        *T = download<double>(r.T.v);
        if (frank) *frank = r.frank;
        end_call(t0);
    });
}

void id_rand_decomp_fixed_rank(mat *M, rsvd_int k, rsvd_int p, rsvd_int q, rsvd_int s, vec **I, mat **T) {
    *I = nullptr;
    *T = nullptr;
    guarded("id_rand_decomp_fixed_rank", [&] {
        check_mat(M);
        need_int(k, p, q, s);
        need(k >= 1 && p >= 0 && k + p <= std::min(M->nrows, M->ncols), "need 1 <= k, k + p <= min(m, n)");
        need(q < 1 || s >= 1, "s must be >= 1");
        begin_call();
        auto t0 = Clock::now();
        DMat<double> A = upload<double>(M);
        IdOut r = id_rand(A.v, k, p, q, s);
        *I = index_vec(r.I);
        *T = download<double>(r.T.v);
        end_call(t0);
    });
}

void id_blockrand_decomp_fixed_rank_or_prec(mat *M, rsvd_int k, rsvd_int p, real TOL, rsvd_int kstep, rsvd_int q, rsvd_int s, rsvd_int *frank,
                                            vec **I, mat **T) {
    *I = nullptr;
    *T = nullptr;
    guarded("id_blockrand_decomp_fixed_rank_or_prec", [&] {
        check_mat(M);
        need_int(k, p, kstep, q, s);
        need(kstep >= 1, "need kstep >= 1");
        need(q < 1 || s >= 1, "s must be >= 1");
        begin_call();
        auto t0 = Clock::now();
        DMat<double> A = upload<double>(M);
        IdOut r = id_blockrand(A.v, k, p, TOL, kstep, q, s);
        *I = index_vec(r.I);
        *T = download<double>(r.T.v);
        if (frank) *frank = r.frank;
        end_call(t0);
    });
}

void low_rank_svd_rand_decomp_fromQB(mat *Q, mat *B, mat **U, mat **S, mat **V) {
    *U = *S = *V = nullptr;
    guarded("low_rank_svd_rand_decomp_fromQB", [&] {
        check_mat(Q);
        check_mat(B);
        need(Q->ncols == B->nrows, "Q must have as many columns as B has rows");
        begin_call();
        auto t0 = Clock::now();
        DMat<double> dQ = upload<double>(Q), dB = upload<double>(B);
        SvdOut<double> r = svd_from_qb(dQ.v, dB.v);
        svd_outputs<double>(r, U, S, V);
        end_call(t0);
    });
}

void id_rand_decomp_fromQB(mat *Q, mat *B, vec **I, mat **T) {
    *I = nullptr;
    *T = nullptr;
    guarded("id_rand_decomp_fromQB", [&] {
        check_mat(Q);
        check_mat(B);
        need(Q->ncols <= std::min(B->nrows, B->ncols), "Q->ncols must not exceed min(B rows, B cols)");
        begin_call();
        auto t0 = Clock::now();
        DMat<double> dB = upload<double>(B);
        IdOut r = id_from_qb(dB.v, Q->ncols);
        *I = index_vec(r.I);
        *T = download<double>(r.T.v);
        end_call(t0);
    });
}

// ---- the older randomized SVD entry points (RRA:385-700).  Each is one of the entry points above
// with fixed parameters -- identities that hold bit for bit on the reference's own build:
// svd1 = the fixed-rank rSVD with p = 0, vnum = 2 (eig of B B^T, ascending), no power round;
// svd2 = the same with vnum = 1 (QR of B^T, descending); svd3 = vnum = 1 with q, s;
// svd4 = randQB_pb (kstep, nstep, p power rounds, s = 1) then the eig(B B^T) back end, ascending.
void randomized_low_rank_svd1(mat *M, rsvd_int k, mat **U, mat **S, mat **V) {
    low_rank_svd_rand_decomp_fixed_rank(M, k, 0, 2, 1, 1, nullptr, U, S, V);
}
void randomized_low_rank_svd2(mat *M, rsvd_int k, mat **U, mat **S, mat **V) {
    low_rank_svd_rand_decomp_fixed_rank(M, k, 0, 1, 1, 1, nullptr, U, S, V);
}
void randomized_low_rank_svd3(mat *M, rsvd_int k, rsvd_int q, rsvd_int s, mat **U, mat **S, mat **V) {
    low_rank_svd_rand_decomp_fixed_rank(M, k, 0, 1, q, s, nullptr, U, S, V);
}
void randomized_low_rank_svd4(mat *M, rsvd_int kstep, rsvd_int nstep, rsvd_int p, mat **U, mat **S, mat **V) {
    *U = *S = *V = nullptr;
    mat *Q = nullptr, *B = nullptr;
    randQB_pb(M, kstep, nstep, p, 1, &Q, &B);
    if (!Q || !B) return;                                // rsvdpack_last_error() says why
    low_rank_svd_rand_decomp_fromQB(Q, B, U, S, V);
    matrix_delete(Q);
    matrix_delete(B);
    if (!*U || !*S || !*V) return;
    // the QB split returns the pairs descending; this entry point returns them ascending
    auto reverse_cols = [](mat *X) {
        for (rsvd_int a = 0, b = X->ncols - 1; a < b; a++, b--)
            std::swap_ranges(X->d + (size_t)a * X->nrows, X->d + (size_t)(a + 1) * X->nrows, X->d + (size_t)b * X->nrows);
    };
    reverse_cols(*U);
    reverse_cols(*V);
    const rsvd_int l = (*S)->nrows;
    for (rsvd_int a = 0, b = l - 1; a < b; a++, b--)
        std::swap((*S)->d[(size_t)a * l + a], (*S)->d[(size_t)b * l + b]);
}

static void two_sided_outputs(TwoSidedOut &r, vec **Icol, vec **Irow, mat **T, mat **S) {
    *Icol = index_vec(r.Icol);
    *Irow = index_vec(r.Irow);
    *T = download<double>(r.T.v);
    *S = download<double>(r.S.v);
}

void id_two_sided_decomp_fixed_rank_or_prec(mat *M, rsvd_int k, real TOL, rsvd_int *frank, vec **Icol, vec **Irow, mat **T,
                                            mat **S) {
    *Icol = *Irow = nullptr;
    *T = *S = nullptr;
    guarded("id_two_sided_decomp_fixed_rank_or_prec", [&] {
        check_mat(M);
        need_int(k);
        need(k <= std::min(M->nrows, M->ncols), "k exceeds min(m, n)");
        begin_call();
        auto t0 = Clock::now();
        DMat<double> A = upload<double>(M);
        TwoSidedOut r = id_two_sided(A.v, id_det(A.v, k, TOL));
        two_sided_outputs(r, Icol, Irow, T, S);
        if (frank) *frank = r.frank;
        end_call(t0);
    });
}

void id_two_sided_rand_decomp_fixed_rank(mat *M, rsvd_int k, rsvd_int p, rsvd_int q, rsvd_int s, vec **Icol, vec **Irow, mat **T,
                                         mat **S) {
    *Icol = *Irow = nullptr;
    *T = *S = nullptr;
    guarded("id_two_sided_rand_decomp_fixed_rank", [&] {
        check_mat(M);
        need_int(k, p, q, s);
        need(k >= 1 && p >= 0 && k + p <= std::min(M->nrows, M->ncols), "need 1 <= k, k + p <= min(m, n)");
        need(q < 1 || s >= 1, "s must be >= 1");
        begin_call();
        auto t0 = Clock::now();
        DMat<double> A = upload<double>(M);
        TwoSidedOut r = id_two_sided(A.v, id_rand(A.v, k, p, q, s));
        two_sided_outputs(r, Icol, Irow, T, S);
        end_call(t0);
    });
}

void id_two_sided_blockrand_decomp_fixed_rank_or_prec(mat *M, rsvd_int k, rsvd_int p, real TOL, rsvd_int kstep, rsvd_int q, rsvd_int s,
                                                      rsvd_int *frank, vec **Icol, vec **Irow, mat **T, mat **S) {
    *Icol = *Irow = nullptr;
    *T = *S = nullptr;
    guarded("id_two_sided_blockrand_decomp_fixed_rank_or_prec", [&] {
        check_mat(M);
        need_int(k, p, kstep, q, s);
        need(kstep >= 1, "need kstep >= 1");
        need(q < 1 || s >= 1, "s must be >= 1");
        begin_call();
        auto t0 = Clock::now();
        DMat<double> A = upload<double>(M);
        TwoSidedOut r = id_two_sided(A.v, id_blockrand(A.v, k, p, TOL, kstep, q, s));
        two_sided_outputs(r, Icol, Irow, T, S);
        if (frank) *frank = r.frank;
        end_call(t0);
    });
}

static void cur_outputs(CurOut &r, mat **C, mat **U, mat **R) {
    *C = download<double>(r.C.v);
    *U = download<double>(r.U.v);
    *R = download<double>(r.R.v);
}

void cur_decomp_fixed_rank_or_prec(mat *M, rsvd_int k, real TOL, rsvd_int *frank, mat **C, mat **U, mat **R) {
    *C = *U = *R = nullptr;
    guarded("cur_decomp_fixed_rank_or_prec", [&] {
        check_mat(M);
        need_int(k);
        need(k <= std::min(M->nrows, M->ncols), "k exceeds min(m, n)");
        begin_call();
        auto t0 = Clock::now();
        DMat<double> A = upload<double>(M);
        TwoSidedOut ts = id_two_sided(A.v, id_det(A.v, k, TOL));
        CurOut r = cur_from_two_sided(A.v, ts.frank, ts);
        cur_outputs(r, C, U, R);
        if (frank) *frank = ts.frank;
        end_call(t0);
    });
}

void cur_rand_decomp_fixed_rank(mat *M, rsvd_int k, rsvd_int p, rsvd_int q, rsvd_int s, mat **C, mat **U, mat **R) {
    *C = *U = *R = nullptr;
    guarded("cur_rand_decomp_fixed_rank", [&] {
        check_mat(M);
        need_int(k, p, q, s);
        need(k >= 1 && p >= 0 && k + p <= std::min(M->nrows, M->ncols), "need 1 <= k, k + p <= min(m, n)");
        need(q < 1 || s >= 1, "s must be >= 1");
        begin_call();
        auto t0 = Clock::now();
        DMat<double> A = upload<double>(M);
        TwoSidedOut ts = id_two_sided(A.v, id_rand(A.v, k, p, q, s));
        CurOut r = cur_from_two_sided(A.v, k, ts);
        cur_outputs(r, C, U, R);
        end_call(t0);
    });
}

void cur_blockrand_decomp_fixed_rank_or_prec(mat *M, rsvd_int k, rsvd_int p, real TOL, rsvd_int kstep, rsvd_int q, rsvd_int s, rsvd_int *frank,
                                             mat **C, mat **U, mat **R) {
    *C = *U = *R = nullptr;
    guarded("cur_blockrand_decomp_fixed_rank_or_prec", [&] {
        check_mat(M);
        need_int(k, p, kstep, q, s);
        need(kstep >= 1, "need kstep >= 1");
        need(q < 1 || s >= 1, "s must be >= 1");
        begin_call();
        auto t0 = Clock::now();
        DMat<double> A = upload<double>(M);
        TwoSidedOut ts = id_two_sided(A.v, id_blockrand(A.v, k, p, TOL, kstep, q, s));
        CurOut r = cur_from_two_sided(A.v, ts.frank, ts);
        cur_outputs(r, C, U, R);
        if (frank) *frank = ts.frank;
        end_call(t0);
    });
}

// ============================================================ device-resident entry points
}  // extern "C"
template <typename T>
static void dev_svd(const void *dA, long long lda, int m, int n, int k, int p, int vnum, int q, int s, void *dU,
                    long long ldu, double *dS, void *dV, long long ldv) {
    cudaStream_t st = ctx().stream;
    DM<T> A{(T *)const_cast<void *>(dA), m, n, lda};
    SvdOut<T> r = svd_fixed_rank<T>(A, k, p, vnum, q, s);
    RSVD_CK(cudaMemcpy2DAsync(dU, sizeof(T) * ldu, r.U.v.p, sizeof(T) * r.U.v.ld, sizeof(T) * m, k,
                              cudaMemcpyDeviceToDevice, st));
    RSVD_CK(cudaMemcpy2DAsync(dV, sizeof(T) * ldv, r.V.v.p, sizeof(T) * r.V.v.ld, sizeof(T) * n, k,
                              cudaMemcpyDeviceToDevice, st));
    RSVD_CK(cudaMemcpyAsync(dS, r.S.data(), sizeof(double) * k, cudaMemcpyHostToDevice, st));
    RSVD_CK(cudaStreamSynchronize(st));
}
extern "C" {

int rsvdpack_dev_svd_fixed_rank(const void *dA, int dtype, long long lda, int m, int n, int k, int p, int vnum,
                                int q, int s, void *dU, long long ldu, double *dS, void *dV, long long ldv) {
    guarded("rsvdpack_dev_svd_fixed_rank", [&] {
        need(dA && dU && dS && dV, "null device pointer");
        need(m > 0 && n > 0 && k >= 1 && p >= 0 && k + p <= std::min(m, n), "bad sizes");
        need(lda >= m && ldu >= m && ldv >= n, "bad leading dimension");
        need(q < 2 || s >= 1, "s must be >= 1 when q >= 2");
        begin_call();
        order_after_default_stream();
        auto t0 = Clock::now();
        if (dtype == RSVD_DT_F64) dev_svd<double>(dA, lda, m, n, k, p, vnum, q, s, dU, ldu, dS, dV, ldv);
        else if (dtype == RSVD_DT_F32) dev_svd<float>(dA, lda, m, n, k, p, vnum, q, s, dU, ldu, dS, dV, ldv);
        else fail(RSVD_ERR_ARGUMENT, "unknown dtype");
        end_call(t0);
    });
    return rsvdpack_last_error();
}

int rsvdpack_dev_sketch(const void *dA, int dtype, long long lda, int m, int n, const void *dX, long long ldx, int w,
                        void *dY, long long ldy, int trans) {
    guarded("rsvdpack_dev_sketch", [&] {
        need(dA && dX && dY, "null device pointer");
        need(m > 0 && n > 0 && w > 0 && lda >= m, "bad sizes");
        begin_call();
        order_after_default_stream();
        cudaStream_t st = ctx().stream;
        const i64 xr = trans ? m : n, yr = trans ? n : m;
        need(ldx >= xr && ldy >= yr, "bad leading dimension");
        // device time of the product itself (events on the engine stream) -> timing.sketch_ms
        thread_local cudaEvent_t ev[2] = {nullptr, nullptr};
        for (auto &e : ev)
            if (!e) RSVD_CK(cudaEventCreate(&e));
        if (dtype == RSVD_DT_F64) {
            DM<double> A{(double *)const_cast<void *>(dA), m, n, lda}, X{(double *)const_cast<void *>(dX), xr, w, ldx};
            DM<double> Y{(double *)dY, yr, w, ldy};
            RSVD_CK(cudaEventRecord(ev[0], st));
            prod<double>(st, trans != 0, false, 1.0, A, X, 0.0, Y);
        } else if (dtype == RSVD_DT_F32) {
            DM<float> A{(float *)const_cast<void *>(dA), m, n, lda}, X{(float *)const_cast<void *>(dX), xr, w, ldx};
            DM<float> Y{(float *)dY, yr, w, ldy};
            RSVD_CK(cudaEventRecord(ev[0], st));
            prod<float>(st, trans != 0, false, 1.0f, A, X, 0.0f, Y);
        } else if (dtype == RSVD_DT_BF16) {
            // BF16-resident A: one kind::f16 tensor-core product on X rounded to BF16
            need(((uintptr_t)dA % 16 == 0) && (lda * 2) % 16 == 0, "BF16 A must be 16-byte aligned, lda % 8 == 0");
            DM<float> X{(float *)const_cast<void *>(dX), xr, w, ldx};
            DMat<__nv_bfloat16> Xb(xr, w, st, false);
            convert<float, __nv_bfloat16>(st, X, Xb.v);
            RSVD_CK(cudaEventRecord(ev[0], st));
            tc_gemm(st, 1, trans == 0, dA, lda, Xb.v.p, Xb.v.ld, (int)yr, w, (int)xr, 1.0f, (float *)dY, ldy, 0,
                    nullptr, 0, nullptr, 0);
        } else {
            fail(RSVD_ERR_ARGUMENT, "unknown dtype");
        }
        RSVD_CK(cudaEventRecord(ev[1], st));
        RSVD_CK(cudaStreamSynchronize(st));
        float ms = 0.f;
        RSVD_CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
        ctx().timing.sketch_ms = ms;
        release_operand_cache();
        check_device_flags(ctx());
        ctx().timing.kernel_launches = ctx().launches;
    });
    return rsvdpack_last_error();
}

// ---- FP32-accurate tensor-core products (k_gemm_tc.cu: split_tf32, tc_gemm_3xtf32, tc_update_3xtf32)
namespace {
void split_operands(cudaStream_t st, const float *dA, long long lda, const float *dX, long long ldx, int M, int N,
                    int K, DMat<float> &Ah, DMat<float> &Al, DMat<float> &Xh, DMat<float> &Xl) {
    Ah = DMat<float>(K, M, st, false);
    Al = DMat<float>(K, M, st, false);
    Xh = DMat<float>(K, N, st, false);
    Xl = DMat<float>(K, N, st, false);
    split_tf32(st, dA, lda, K, M, Ah.v.p, Al.v.p, Ah.v.ld);
    split_tf32(st, dX, ldx, K, N, Xh.v.p, Xl.v.p, Xh.v.ld);
}
}  // namespace

int rsvdpack_dev_gemm_3xtf32(const float *dA, long long lda, const float *dX, long long ldx, int M, int N, int K,
                             float *dD, long long ldd) {
    guarded("rsvdpack_dev_gemm_3xtf32", [&] {
        need(dA && dX && dD, "null device pointer");
        need(M > 0 && N > 0 && K > 0, "bad sizes");
        need(lda >= K && ldx >= K && ldd >= M, "bad leading dimension");
        begin_call();
        order_after_default_stream();
        cudaStream_t st = ctx().stream;
        DMat<float> Ah, Al, Xh, Xl;
        split_operands(st, dA, lda, dX, ldx, M, N, K, Ah, Al, Xh, Xl);
        tc_gemm_3xtf32(st, Ah.v.p, Al.v.p, Ah.v.ld, Xh.v.p, Xl.v.p, Xh.v.ld, M, N, K, dD, ldd);
        RSVD_CK(cudaStreamSynchronize(st));
        check_device_flags(ctx());
        ctx().timing.kernel_launches = ctx().launches;
    });
    return rsvdpack_last_error();
}

int rsvdpack_dev_residual_norms(const void *dA, int dtype, long long lda, int m, int n, const void *dU,
                                long long ldu, const double *dS, const void *dV, long long ldv, int k, int iters,
                                double *fro, double *spec) {
    guarded("rsvdpack_dev_residual_norms", [&] {
        need(dA && (k == 0 || (dU && dS && dV)), "null device pointer");
        need(m > 0 && n > 0 && k >= 0 && k <= std::min(m, n) && iters >= 0, "bad sizes");
        need(lda >= m && (k == 0 || (ldu >= m && ldv >= n)), "bad leading dimension");
        need(dtype == RSVD_DT_F64 || dtype == RSVD_DT_F32, "dtype must be RSVD_DT_F64 or RSVD_DT_F32");
        begin_call();
        order_after_default_stream();
        if (dtype == RSVD_DT_F64) {
            residual_norms<double>(DM<double>{(double *)dA, m, n, lda}, DM<double>{(double *)dU, m, k, ldu}, dS,
                                   DM<double>{(double *)dV, n, k, ldv}, fro, spec, iters);
        } else {
            residual_norms<float>(DM<float>{(float *)dA, m, n, lda}, DM<float>{(float *)dU, m, k, ldu}, dS,
                                  DM<float>{(float *)dV, n, k, ldv}, fro, spec, iters);
        }
        RSVD_CK(cudaStreamSynchronize(ctx().stream));
        ctx().timing.kernel_launches = ctx().launches;
    });
    return rsvdpack_last_error();
}

int rsvdpack_binary_file_shape(const char *fname, long long *m, long long *n) {
    guarded("rsvdpack_binary_file_shape", [&] {
        need(fname && m && n, "null argument");
        if (!binary_file_shape(fname, (int)sizeof(rsvd_int), m, n))
            fail(RSVD_ERR_ARGUMENT, std::string("cannot read a matrix file header from ") + fname);
    });
    return rsvdpack_last_error();
}

int rsvdpack_dev_load_binary(const char *fname, int dtype, void *dA, long long lda, long long *m, long long *n) {
    guarded("rsvdpack_dev_load_binary", [&] {
        need(fname && dA, "null argument");
        need(dtype == RSVD_DT_F64 || dtype == RSVD_DT_F32 || dtype == RSVD_DT_BF16,
             "dtype must be RSVD_DT_F64, RSVD_DT_F32 or RSVD_DT_BF16");
        begin_call();
        order_after_default_stream();
        long long mm = 0, nn = 0;
        load_binary_to_device(fname, (int)sizeof(rsvd_int), (int)sizeof(real), dtype, dA, lda, &mm, &nn);
        if (m) *m = mm;
        if (n) *n = nn;
        ctx().timing.kernel_launches = ctx().launches;
    });
    return rsvdpack_last_error();
}

int rsvdpack_dev_gemm_df64(int ta, int tb, int M, int N, int K, double alpha, const double *dA, long long lda,
                           const double *dB, long long ldb, double beta, double *dC, long long ldc) {
    guarded("rsvdpack_dev_gemm_df64", [&] {
        need(dA && dB && dC, "null device pointer");
        need(M > 0 && N > 0 && K > 0, "bad sizes");
        need(lda >= (ta ? K : M) && ldb >= (tb ? N : K) && ldc >= M, "bad leading dimension");
        begin_call();
        order_after_default_stream();
        cudaStream_t st = ctx().stream;
        DM<double> A{const_cast<double *>(dA), ta ? K : M, ta ? M : K, lda};
        DM<double> B{const_cast<double *>(dB), tb ? N : K, tb ? K : N, ldb};
        Df64Split As(st, A), Bs(st, B);
        {
            PhaseTimer pt(&ctx().timing.sketch_ms);
            df64_gemm(st, ta != 0, tb != 0, alpha, As, Bs, beta, DM<double>{dC, M, N, ldc});
        }
        phase_collect();
        ctx().timing.kernel_launches = ctx().launches;
    });
    return rsvdpack_last_error();
}

int rsvdpack_dev_update_3xtf32(const float *dA, long long lda, const float *dX, long long ldx, int M, int N, int K,
                               float *dC, long long ldc, double *fro2) {
    guarded("rsvdpack_dev_update_3xtf32", [&] {
        need(dA && dX && dC, "null device pointer");
        need(M > 0 && N > 0 && K > 0, "bad sizes");
        need(lda >= K && ldx >= K && ldc >= M, "bad leading dimension");
        begin_call();
        order_after_default_stream();
        cudaStream_t st = ctx().stream;
        DMat<float> Ah, Al, Xh, Xl;
        split_operands(st, dA, lda, dX, ldx, M, N, K, Ah, Al, Xh, Xl);
        // one sum of squares per CTA of the update grid (128-row tiles; one column tile up
        // to 512 columns, else 256-column tiles)
        const long long parts = ((long long)M + 127) / 128 * (N <= 512 ? 1 : ((long long)N + 255) / 256);
        DBuf fp(sizeof(double) * (size_t)parts, st);
        tc_update_3xtf32(st, Ah.v.p, Al.v.p, Ah.v.ld, Xh.v.p, Xl.v.p, Xh.v.ld, M, N, K, dC, ldc,
                         fro2 ? (double *)fp.get() : nullptr);
        std::vector<double> h(fro2 ? (size_t)parts : 0);
        if (fro2) RSVD_CK(cudaMemcpyAsync(h.data(), fp.get(), sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st));
        RSVD_CK(cudaStreamSynchronize(st));
        check_device_flags(ctx());
        if (fro2) {
            double acc = 0.0;
            for (double v : h) acc += v;
            *fro2 = acc;
        }
        ctx().timing.kernel_launches = ctx().launches;
    });
    return rsvdpack_last_error();
}

// ---- the learned proposal's network (k_mlp.cu): device pointers, engine stream, synchronous
int rsvdpack_mlp_info(int *dims, int *nparams) {
    guarded("rsvdpack_mlp_info", [&] {
        need(dims && nparams, "null pointer");
        mlp_dims(dims);
        *nparams = mlp_param_count();
    });
    return rsvdpack_last_error();
}

int rsvdpack_dev_qb(const void *dA, int dtype, long long lda, int m, int n, int kstep, int nstep, double TOL, int q,
                    int s, void *dQ, long long ldq, void *dB, long long ldb, int cap, int *frank) {
    guarded("rsvdpack_dev_qb", [&] {
        need(dA && dQ && dB && frank, "null pointer");
        need(m > 0 && n > 0 && lda >= m && ldq >= m && kstep > 0 && q >= 0 && s >= 1 && cap > 0 && ldb >= cap,
             "bad sizes");
        auto t0 = Clock::now();
        begin_call();
        order_after_default_stream();
        cudaStream_t st = ctx().stream;
        auto run = [&](auto tag) {
            using T = decltype(tag);
            DM<T> A{(T *)const_cast<void *>(dA), m, n, lda};
            QBOut<T> r = qb_blocked<T>(A, kstep, nstep, TOL, q, s);
            if (r.frank > cap) fail(RSVD_ERR_ARGUMENT, "rsvdpack_dev_qb: rank above the output capacity");
            *frank = r.frank;
            if (r.frank > 0) {
                RSVD_CK(cudaMemcpy2DAsync(dQ, sizeof(T) * ldq, r.Q.v.p, sizeof(T) * r.Q.v.ld, sizeof(T) * m, r.frank,
                                          cudaMemcpyDeviceToDevice, st));
                RSVD_CK(cudaMemcpy2DAsync(dB, sizeof(T) * ldb, r.B.v.p, sizeof(T) * r.B.v.ld, sizeof(T) * r.frank, n,
                                          cudaMemcpyDeviceToDevice, st));
            }
            RSVD_CK(cudaStreamSynchronize(st));
        };
        if (dtype == RSVD_DT_F64) run(double{});
        else if (dtype == RSVD_DT_F32) run(float{});
        else fail(RSVD_ERR_ARGUMENT, "unknown dtype");
        end_call(t0);
    });
    return rsvdpack_last_error();
}

int rsvdpack_set_proposal_model(const float *params, int nparams, const float *norm, int nnorm, const float *margin,
                                int nmargin) {
    guarded("rsvdpack_set_proposal_model", [&] {
        int dims[4];
        mlp_dims(dims);
        need(params && norm && margin, "null pointer");
        need(nparams == mlp_param_count(), "parameter count does not match the network");
        need(nnorm == 2 * dims[0] && nmargin == dims[3], "norm / margin length does not match the network");
        ProposalModel m;
        m.params.assign(params, params + nparams);
        m.norm.assign(norm, norm + nnorm);
        m.margin.assign(margin, margin + nmargin);
        set_proposal_model(std::move(m));
    });
    return rsvdpack_last_error();
}

int rsvdpack_load_proposal_model(const char *path) {
    guarded("rsvdpack_load_proposal_model", [&] {
        need(path != nullptr, "null path");
        FILE *fp = std::fopen(path, "rb");
        if (!fp) fail(RSVD_ERR_ARGUMENT, std::string("cannot open ") + path);
        std::vector<float> P, N, M;
        char magic[8];
        int nd = 0, dims[8] = {0}, np = 0, nn = 0;
        bool ok = std::fread(magic, 1, 8, fp) == 8 && std::memcmp(magic, "RSVDMLP1", 8) == 0 &&
                  std::fread(&nd, 4, 1, fp) == 1 && nd >= 2 && nd <= 8 && std::fread(dims, 4, nd, fp) == (size_t)nd &&
                  std::fread(&np, 4, 1, fp) == 1 && std::fread(&nn, 4, 1, fp) == 1 && np > 0 && np < (1 << 24) &&
                  nn > 0 && nn < (1 << 16);
        if (ok) {
            P.resize(np);
            N.resize(nn);
            M.resize(dims[nd - 1]);
            ok = std::fread(P.data(), 4, np, fp) == (size_t)np && std::fread(N.data(), 4, nn, fp) == (size_t)nn &&
                 std::fread(M.data(), 4, M.size(), fp) == M.size();
        }
        std::fclose(fp);
        if (!ok) fail(RSVD_ERR_ARGUMENT, std::string("not a valid RSVDMLP1 weights file: ") + path);
        if (rsvdpack_set_proposal_model(P.data(), np, N.data(), nn, M.data(), (int)M.size()) != RSVD_OK)
            fail(RSVD_ERR_ARGUMENT, "weights file does not match the network");
    });
    return rsvdpack_last_error();
}

int rsvdpack_mlp_forward(const float *dP, const float *dnorm, const float *dX, int batch, float *dY) {
    guarded("rsvdpack_mlp_forward", [&] {
        need(dP && dnorm && dX && dY, "null device pointer");
        need(batch > 0, "empty batch");
        begin_call();
        order_after_default_stream();
        cudaStream_t st = ctx().stream;
        mlp_forward(st, dP, dnorm, dX, batch, dY);
        RSVD_CK(cudaStreamSynchronize(st));
        check_device_flags(ctx());
    });
    return rsvdpack_last_error();
}

int rsvdpack_mlp_train_step(float *dP, float *dM, float *dV, const float *dnorm, const float *dX, const float *dT,
                            const float *dReached, int batch, float lr, int step, float *dloss, float *dG) {
    guarded("rsvdpack_mlp_train_step", [&] {
        need(dP && dnorm && dX && dT && dReached && dloss && dG, "null device pointer");
        need(lr <= 0.f || (dM && dV), "Adam state required when lr > 0");
        need(batch > 0 && step >= 1, "bad batch or step");
        begin_call();
        order_after_default_stream();
        cudaStream_t st = ctx().stream;
        mlp_train_step(st, dP, dM, dV, dnorm, dX, dT, dReached, batch, lr, step, dloss, dG);
        RSVD_CK(cudaStreamSynchronize(st));
        check_device_flags(ctx());
    });
    return rsvdpack_last_error();
}

int rsvdpack_dev_small_svd(double *dG, int n, long long ldg, double *dU, long long ldu, double *dS, double *dV,
                           long long ldv, int fp32) {
    int sweeps = -1;
    guarded("rsvdpack_dev_small_svd", [&] {
        need(dG && dU && dS && dV, "null device pointer");
        need(n > 0 && ldg >= n && ldu >= n && ldv >= n, "bad sizes");
        begin_call();
        order_after_default_stream();
        cudaStream_t st = ctx().stream;
        DM<double> G{dG, n, n, ldg}, U{dU, n, n, ldu}, V{dV, n, n, ldv};
        int *flag = ctx().d_flags + FLAG_JACOBI_NOCONV;
        if (fp32 == 2) {
            // the mixed modes' l x l SVD: FP32 Jacobi, then the FP64-accurate refinement
            sweeps = jacobi_small<float>(st, G, U, V, dS, flag);
            svd_refine(st, G, V, U, dS, REFINE_STEPS);
        } else {
            sweeps = fp32 ? jacobi_small<float>(st, G, U, V, dS, flag) : jacobi_small<double>(st, G, U, V, dS, flag);
        }
        RSVD_CK(cudaStreamSynchronize(st));
    });
    const int e = rsvdpack_last_error();
    return e ? -e : sweeps;
}

int rsvdpack_dev_small_cholesky(double *dG, int n, long long ldg, int fp32) {
    guarded("rsvdpack_dev_small_cholesky", [&] {
        need(dG && n > 0 && ldg >= n, "bad arguments");
        begin_call();
        order_after_default_stream();
        cudaStream_t st = ctx().stream;
        DM<double> G{dG, n, n, ldg};
        int *flag = ctx().d_flags + FLAG_CHOL_BREAKDOWN;
        const bool ok = fp32 ? cholesky_small<float>(st, G, 0.0, flag) : cholesky_small<double>(st, G, 0.0, flag);
        if (!ok) fail(RSVD_ERR_NUMERIC, "Cholesky breakdown (matrix not positive definite)");
    });
    return rsvdpack_last_error();
}

void *rsvdpack_stream(void) {
    try {
        return (void *)ctx().stream;
    } catch (const Error &e) {
        set_error(e.code, e.what());
        return nullptr;
    }
}

// ============================================================ approximation reports (RRA:2337-2573)
void use_low_rank_svd_for_approximation(mat *M, mat *U, mat *S, mat *V) {
    mat *P = matrix_new(M->nrows, M->ncols);
    form_svd_product_matrix(U, S, V, P);
    std::printf("norm(M,fro) = %f\n", get_matrix_frobenius_norm(M));
    std::printf("norm(P,fro) = %f\n", get_matrix_frobenius_norm(P));
    std::printf("percent error = %f\n", get_percent_error_between_two_mats(M, P));
    matrix_delete(P);
}

void use_pivoted_QR_decomp_for_approximation(mat *M, mat *Qk, mat *Rk, vec *I) {
    const rsvd_int m = M->nrows, n = M->ncols;
    mat *QR = matrix_new(m, n), *QRPt = matrix_new(m, n);
    matrix_matrix_mult(Qk, Rk, QR);
    // (Qk Rk) P^T : column j of the product goes back to column I[j]
    for (rsvd_int j = 0; j < n; j++)
        std::memcpy(QRPt->d + (size_t)((rsvd_int)I->d[j]) * m, QR->d + (size_t)j * m, sizeof(real) * m);
    std::printf("percent_error between M and QkRkPt = %f\n", get_percent_error_between_two_mats(M, QRPt));
    matrix_delete(Qk);
    matrix_delete(Rk);
    matrix_delete(QR);
    matrix_delete(QRPt);
}

void use_QB_decomp_for_approximation(mat *M, mat *Q, mat *B) {
    mat *P = matrix_new(M->nrows, M->ncols);
    matrix_matrix_mult(Q, B, P);
    std::printf("norm(M,fro) = %f\n", get_matrix_frobenius_norm(M));
    std::printf("norm(P,fro) = %f\n", get_matrix_frobenius_norm(P));
    std::printf("percent error = %f\n", get_percent_error_between_two_mats(M, P));
    matrix_delete(P);
}

// V = [I_k; T^T](Iinv,:) ; MA = M(:,I(1:k)) V^T
static mat *id_basis(mat *T, vec *I, rsvd_int k) {
    const rsvd_int n = I->nrows;
    std::vector<rsvd_int> inv((size_t)n);
    for (rsvd_int j = 0; j < n; j++) inv[(size_t)((rsvd_int)I->d[j])] = j;
    mat *V = matrix_new(n, k);
    for (rsvd_int i = 0; i < n; i++) {
        const rsvd_int r = inv[(size_t)i];
        for (rsvd_int c = 0; c < k; c++)
            V->d[(size_t)c * n + i] = (r < k) ? (r == c ? 1.0 : 0.0) : T->d[(size_t)(r - k) * T->nrows + c];
    }
    return V;
}

void use_id_decomp_for_approximation(mat *M, mat *T, vec *I, rsvd_int k) {
    const rsvd_int m = M->nrows, n = M->ncols;
    mat *V = id_basis(T, I, k);
    mat *MI = matrix_new(m, k);
    for (rsvd_int c = 0; c < k; c++) std::memcpy(MI->d + (size_t)c * m, M->d + (size_t)((rsvd_int)I->d[c]) * m, sizeof(real) * m);
    mat *MA = matrix_new(m, n);
    matrix_matrix_transpose_mult(MI, V, MA);
    std::printf("norm(M,fro) = %f\n", get_matrix_frobenius_norm(M));
    std::printf("norm(MA,fro) = %f\n", get_matrix_frobenius_norm(MA));
    std::printf("percent error = %f\n", get_percent_error_between_two_mats(M, MA));
    matrix_delete(V);
    matrix_delete(MI);
    matrix_delete(MA);
}

void use_id_two_sided_decomp_for_approximation(mat *M, mat *T, mat *S, vec *Icol, vec *Irow, rsvd_int k) {
    const rsvd_int m = M->nrows, n = M->ncols;
    mat *V = id_basis(T, Icol, k);
    mat *Uu = id_basis(S, Irow, k);
    mat *MIJ = matrix_new(k, k);
    for (rsvd_int c = 0; c < k; c++)
        for (rsvd_int r = 0; r < k; r++)
            MIJ->d[(size_t)c * k + r] = M->d[(size_t)((rsvd_int)Icol->d[c]) * m + (size_t)((rsvd_int)Irow->d[r])];
    mat *UM = matrix_new(m, k), *MA = matrix_new(m, n);
    matrix_matrix_mult(Uu, MIJ, UM);
    matrix_matrix_transpose_mult(UM, V, MA);
    std::printf("norm(M,fro) = %f\n", get_matrix_frobenius_norm(M));
    std::printf("norm(MA,fro) = %f\n", get_matrix_frobenius_norm(MA));
    std::printf("percent error = %f\n", get_percent_error_between_two_mats(M, MA));
    matrix_delete(V);
    matrix_delete(Uu);
    matrix_delete(MIJ);
    matrix_delete(UM);
    matrix_delete(MA);
}

void use_cur_decomp_for_approximation(mat *M, mat *C, mat *U, mat *R) {
    mat *P = matrix_new(M->nrows, M->ncols);
    form_cur_product_matrix(C, U, R, P);
    std::printf("norm(M,fro) = %f\n", get_matrix_frobenius_norm(M));
    std::printf("norm(P,fro) = %f\n", get_matrix_frobenius_norm(P));
    std::printf("percent error = %f\n", get_percent_error_between_two_mats(M, P));
    matrix_delete(P);
}

}  // extern "C"
