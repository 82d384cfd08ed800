// runtime.cu -- per-thread CUDA context, error state, stream-ordered buffers, engine
// options and the Gaussian test-matrix provider of librsvdpack.
#include "rsvd_internal.h"
#include "k_common.cuh"

#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>

namespace rsvd {

// ------------------------------------------------------------------ errors
namespace {
thread_local int t_err = RSVD_OK;
thread_local std::string t_msg;
}  // namespace

void set_error(int code, const std::string &msg) {
    t_err = code;
    t_msg = msg;
    if (std::getenv("RSVDPACK_DEBUG")) std::fprintf(stderr, "rsvdpack: error %d: %s\n", code, msg.c_str());
}

[[noreturn]] void throw_cuda(cudaError_t e, const char *what, const char *file, int line) {
    char buf[512];
    std::snprintf(buf, sizeof buf, "%s: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    throw Error(e == cudaErrorMemoryAllocation ? RSVD_ERR_ALLOC : RSVD_ERR_CUDA, buf);
}

[[noreturn]] void fail(int code, const std::string &msg) { throw Error(code, msg); }

// ------------------------------------------------------------------ options
namespace {
std::mutex g_opts_mu;
bool g_opts_init = false;
rsvdpack_opts g_opts;

void init_opts_locked() {
    if (g_opts_init) return;
    std::memset(&g_opts, 0, sizeof g_opts);
    g_opts.precision = api_default_precision();   // FP64; FP32 in the float-data library
    g_opts.use_provider = 1;
    g_opts.seed = 0x5EED5EEDull;
    g_opts.verbose = 0;
    if (const char *p = std::getenv("RSVDPACK_PRECISION")) {
        std::string v(p);
        if (v == "fp32") g_opts.precision = RSVD_PREC_FP32;
        else if (v == "tf32") g_opts.precision = RSVD_PREC_TF32;
        else if (v == "bf16") g_opts.precision = RSVD_PREC_BF16;
        else if (v == "fp64x") g_opts.precision = RSVD_PREC_FP64X;
    }
    if (const char *p = std::getenv("RSVDPACK_SEED")) g_opts.seed = std::strtoull(p, nullptr, 0);
    if (std::getenv("RSVDPACK_VERBOSE")) g_opts.verbose = 1;
    g_opts_init = true;
}
}  // namespace

const rsvdpack_opts &global_opts() {
    std::lock_guard<std::mutex> g(g_opts_mu);
    init_opts_locked();
    return g_opts;
}

namespace {
std::mutex g_model_mu;
std::unique_ptr<ProposalModel> g_model;
}  // namespace

const ProposalModel *proposal_model() {
    std::lock_guard<std::mutex> g(g_model_mu);
    return g_model.get();
}
void set_proposal_model(ProposalModel m) {
    std::lock_guard<std::mutex> g(g_model_mu);
    g_model.reset(new ProposalModel(std::move(m)));
}

// ------------------------------------------------------------------ provider
namespace {
std::mutex g_prov_mu;
rsvd_omega_fn g_prov = nullptr;
void *g_prov_ctx = nullptr;
int g_prov_calls = 0;
}  // namespace

namespace {
thread_local unsigned long long t_philox_calls = 0;
}
unsigned long long &philox_calls() { return t_philox_calls; }

bool omega_provider_active() {
    std::lock_guard<std::mutex> g(g_prov_mu);
    return g_prov != nullptr;
}

void omega_fill_host(int nrows, int ncols, double *out) {
    std::lock_guard<std::mutex> g(g_prov_mu);
    if (!g_prov) fail(RSVD_ERR_ARGUMENT, "no test-matrix provider registered");
    g_prov(g_prov_ctx, g_prov_calls, nrows, ncols, out);
    g_prov_calls++;
    const size_t n = (size_t)nrows * (size_t)ncols;
    for (size_t i = 0; i < n; i++) out[i] = (double)(float)out[i];   // float Gaussians, as the reference
}

// ------------------------------------------------------------------ context
namespace {
struct CtxHolder {
    Ctx c;
    bool init = false;
    ~CtxHolder() {
        // Streams and buffers die with the CUDA context at process exit; nothing to do.
    }
};
thread_local CtxHolder t_ctx;
}  // namespace

Ctx &ctx() {
    CtxHolder &h = t_ctx;
    if (h.init) return h.c;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        fail(RSVD_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    }
    int dev = 0;
    if (const char *p = std::getenv("RSVDPACK_DEVICE")) dev = std::atoi(p);
    RSVD_CK(cudaSetDevice(dev));
    cudaDeviceProp prop;
    RSVD_CK(cudaGetDeviceProperties(&prop, dev));
    if (!(prop.major == 10 && prop.minor == 3))
        fail(RSVD_ERR_NO_DEVICE, std::string("librsvdpack is built for sm_103a (GB300); found ") + prop.name);
    h.c.device = dev;
    h.c.sms = prop.multiProcessorCount;
    h.c.cc_major = prop.major;
    h.c.cc_minor = prop.minor;
    int pma = 0;
    if (cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
        cudaGetLastError();
        pma = 0;
    }
    h.c.pageable_access = pma != 0;
    RSVD_CK(cudaStreamCreateWithFlags(&h.c.stream, cudaStreamNonBlocking));
    cudaMemPool_t pool;
    RSVD_CK(cudaDeviceGetDefaultMemPool(&pool, dev));
    unsigned long long thr = ~0ull;
    RSVD_CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
    RSVD_CK(cudaMalloc(&h.c.d_flags, sizeof(int) * FLAG_COUNT));
    RSVD_CK(cudaMemset(h.c.d_flags, 0, sizeof(int) * FLAG_COUNT));
    h.init = true;
    return h.c;
}

namespace {
cudaEvent_t pooled_event(Ctx &c) {
    if (c.ev_used == c.ev_pool.size()) {
        cudaEvent_t e;
        RSVD_CK(cudaEventCreate(&e));
        c.ev_pool.push_back(e);
    }
    return c.ev_pool[c.ev_used++];
}
}  // namespace

PhaseTimer::PhaseTimer(double *acc_ms) : acc(acc_ms) {
    Ctx &c = ctx();
    cudaEvent_t a = pooled_event(c);
    b = pooled_event(c);
    RSVD_CK(cudaEventRecord(a, c.stream));
    c.marks.push_back({a, b, acc});
}
PhaseTimer::~PhaseTimer() {
    Ctx &c = ctx();
    cudaEventRecord(b, c.stream);           // no throw from a destructor; errors surface later
}
void phase_reset() {
    Ctx &c = ctx();
    c.marks.clear();
    c.ev_used = 0;
}
void phase_collect() {
    Ctx &c = ctx();
    if (c.marks.empty()) return;
    RSVD_CK(cudaStreamSynchronize(c.stream));
    for (auto &mk : c.marks) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, mk.a, mk.b) == cudaSuccess) *mk.acc += ms;
        else cudaGetLastError();
    }
    c.marks.clear();
    c.ev_used = 0;
}

void check_device_flags(Ctx &c) {
    int f[FLAG_COUNT];
    RSVD_CK(cudaMemcpyAsync(f, c.d_flags, sizeof f, cudaMemcpyDeviceToHost, c.stream));
    RSVD_CK(cudaStreamSynchronize(c.stream));
    if (f[FLAG_TIMEOUT]) {
        RSVD_CK(cudaMemsetAsync(c.d_flags, 0, sizeof f, c.stream));
        fail(RSVD_ERR_TIMEOUT, "a bounded device-side wait gave up");
    }
}

// ------------------------------------------------------------------ buffers
DBuf::DBuf(size_t bytes, cudaStream_t s) : n_(bytes), s_(s) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMallocAsync(&p_, bytes, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        p_ = nullptr;
        char buf[128];
        std::snprintf(buf, sizeof buf, "device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        throw Error(RSVD_ERR_ALLOC, buf);
    }
}
DBuf::~DBuf() {
    if (p_) cudaFreeAsync(p_, s_);
}
DBuf &DBuf::operator=(DBuf &&o) noexcept {
    if (this != &o) {
        if (p_) cudaFreeAsync(p_, s_);
        p_ = o.p_; n_ = o.n_; s_ = o.s_;
        o.p_ = nullptr; o.n_ = 0;
    }
    return *this;
}

template <typename T>
DMat<T>::DMat(i64 r, i64 c, cudaStream_t s, bool zero)
    : buf(sizeof(T) * (size_t)std::max<i64>(1, pad_ld(r)) * (size_t)std::max<i64>(1, c), s) {
    v.p = (T *)buf.get();
    v.r = r;
    v.c = c;
    v.ld = std::max<i64>(1, pad_ld(r));
    if (zero) RSVD_CK(cudaMemsetAsync(v.p, 0, buf.bytes() ? sizeof(T) * (size_t)v.ld * (size_t)std::max<i64>(1, c) : 0, s));
}
template struct DMat<double>;
template struct DMat<float>;
template struct DMat<__nv_bfloat16>;
template struct DMat<int>;

}  // namespace rsvd

// ------------------------------------------------------------------ C ABI: extensions
using namespace rsvd;

extern "C" {

int rsvdpack_last_error(void) { return t_err; }
const char *rsvdpack_last_error_string(void) { return t_msg.c_str(); }
void rsvdpack_clear_error(void) { t_err = RSVD_OK; t_msg.clear(); }

void rsvdpack_get_opts(rsvdpack_opts *opts) {
    if (!opts) return;
    std::lock_guard<std::mutex> g(g_opts_mu);
    init_opts_locked();
    *opts = g_opts;
}

void rsvdpack_set_opts(const rsvdpack_opts *opts) {
    if (!opts) return;
    std::lock_guard<std::mutex> g(g_opts_mu);
    init_opts_locked();
    if (opts->precision < RSVD_PREC_FP64 || opts->precision > RSVD_PREC_FP64X) {
        set_error(RSVD_ERR_ARGUMENT, "rsvdpack_set_opts: unknown precision");
        return;
    }
    g_opts = *opts;
}

void rsvdpack_set_omega_provider(rsvd_omega_fn fn, void *c) {
    std::lock_guard<std::mutex> g(g_prov_mu);
    g_prov = fn;
    g_prov_ctx = c;
    g_prov_calls = 0;
}
void rsvdpack_reset_omega_counter(void) {
    std::lock_guard<std::mutex> g(g_prov_mu);
    g_prov_calls = 0;
    t_philox_calls = 0;
}
int rsvdpack_omega_calls(void) {
    std::lock_guard<std::mutex> g(g_prov_mu);
    return g_prov_calls;
}

int rsvdpack_device_info(char *name, int name_len, int *cc_major, int *cc_minor) {
    try {
        Ctx &c = ctx();
        cudaDeviceProp prop;
        RSVD_CK(cudaGetDeviceProperties(&prop, c.device));
        if (name && name_len > 0) {
            std::strncpy(name, prop.name, (size_t)name_len - 1);
            name[name_len - 1] = 0;
        }
        if (cc_major) *cc_major = prop.major;
        if (cc_minor) *cc_minor = prop.minor;
        return c.sms;
    } catch (const Error &e) {
        set_error(e.code, e.what());
        return -1;
    }
}

void rsvdpack_last_timing(rsvdpack_timing *t) {
    if (!t) return;
    try {
        *t = ctx().timing;
    } catch (const Error &) {
        std::memset(t, 0, sizeof *t);
    }
}

}  // extern "C"
