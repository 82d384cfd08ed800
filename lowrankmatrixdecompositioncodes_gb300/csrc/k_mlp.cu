// k_mlp.cu -- the learned rank / power-count proposal: a small MLP (36 -> 64 -> 64 -> 2,
// ReLU) with hand-written forward, backward and Adam kernels, and its C ABI.
//
// Parameters live in one flat FP32 array, layer by layer: W_l (in x out, row-major) then
// b_l (out).  Inputs are normalised in the first layer: x' = (x - mean) * inv_std (norm =
// [mean(36), inv_std(36)]).  Outputs: predicted log2(width / 32) of the single-shot range
// finder for q = 1 and q = 2 power iterations.
//
// Loss (per output): (y - t)^2 when the training run reached the tolerance within the
// width cap, max(0, t - y)^2 when it did not (the cap is a lower bound there); averaged
// over batch x outputs.
#include "rsvd_internal.h"
#include "k_common.cuh"

#include <cstring>
#include <vector>

namespace rsvd {

namespace {

constexpr int NL = 3;
constexpr int DIMS[NL + 1] = {36, 64, 64, 2};

int param_count() {
    int c = 0;
    for (int l = 0; l < NL; l++) c += DIMS[l] * DIMS[l + 1] + DIMS[l + 1];
    return c;
}
int w_off(int l) {
    int c = 0;
    for (int j = 0; j < l; j++) c += DIMS[j] * DIMS[j + 1] + DIMS[j + 1];
    return c;
}

// Y (B x out) = act(X' W + b), X' = X normalised when norm != null (first layer only)
__global__ void mlp_fwd_kernel(const float *X, int in, const float *W, const float *b, const float *norm, float *Y,
                               int out, int B, int relu) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= B * out) return;
    const int r = t / out, o = t % out;
    float acc = b[o];
    for (int i = 0; i < in; i++) {
        float x = X[(size_t)r * in + i];
        if (norm) x = (x - norm[i]) * norm[in + i];
        acc = fmaf(x, W[(size_t)i * out + o], acc);
    }
    Y[t] = relu ? fmaxf(acc, 0.f) : acc;
}

// dY = d loss / d Y and the loss sum (atomic, FP32)
__global__ void mlp_loss_kernel(const float *Y, const float *T, const float *reached, int n, float inv_count,
                                float *dY, float *loss) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    float d = Y[t] - T[t];
    if (reached[t] == 0.f && d > 0.f) d = 0.f;          // capped target: only too-small predictions cost
    dY[t] = 2.f * d * inv_count;
    atomicAdd(loss, d * d * inv_count);
}

// dZ = dY * act'(Z) (in place on dY), act = ReLU when relu (Yact is the post-activation)
__global__ void mlp_dz_kernel(float *dY, const float *Yact, int n, int relu) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    if (relu && !(Yact[t] > 0.f)) dY[t] = 0.f;
}

// dW (in x out) = X'^T dZ, db = column sums of dZ (one thread per weight / bias)
__global__ void mlp_dw_kernel(const float *X, int in, const float *norm, const float *dZ, int out, int B, float *dW,
                              float *db) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < in * out) {
        const int i = t / out, o = t % out;
        float acc = 0.f;
        for (int r = 0; r < B; r++) {
            float x = X[(size_t)r * in + i];
            if (norm) x = (x - norm[i]) * norm[in + i];
            acc = fmaf(x, dZ[(size_t)r * out + o], acc);
        }
        dW[t] = acc;
    } else if (t < in * out + out) {
        const int o = t - in * out;
        float acc = 0.f;
        for (int r = 0; r < B; r++) acc += dZ[(size_t)r * out + o];
        db[o] = acc;
    }
}

// dX (B x in) = dZ W^T
__global__ void mlp_dx_kernel(const float *dZ, int out, const float *W, int in, int B, float *dX) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= B * in) return;
    const int r = t / in, i = t % in;
    float acc = 0.f;
    for (int o = 0; o < out; o++) acc = fmaf(dZ[(size_t)r * out + o], W[(size_t)i * out + o], acc);
    dX[t] = acc;
}

// Adam (Kingma & Ba 2015), bias-corrected, step t >= 1
__global__ void adam_kernel(float *P, const float *G, float *M, float *V, int n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float g = G[t];
    const float m = b1 * M[t] + (1.f - b1) * g;
    const float v = b2 * V[t] + (1.f - b2) * g * g;
    M[t] = m;
    V[t] = v;
    P[t] -= lr * (m * c1) / (sqrtf(v * c2) + eps);
}

unsigned blocks_for(long long n) { return (unsigned)((n + 255) / 256); }

// forward through all layers; acts[l] (B x DIMS[l+1]) receive the post-activation outputs
void forward(cudaStream_t s, const float *P, const float *norm, const float *X, int B, float *const *acts) {
    const float *in = X;
    for (int l = 0; l < NL; l++) {
        const float *W = P + w_off(l), *b = W + DIMS[l] * DIMS[l + 1];
        const int relu = (l < NL - 1);
        mlp_fwd_kernel<<<blocks_for((long long)B * DIMS[l + 1]), 256, 0, s>>>(in, DIMS[l], W, b, l == 0 ? norm : nullptr,
                                                                              acts[l], DIMS[l + 1], B, relu);
        in = acts[l];
    }
    RSVD_LAUNCH_CK();
    ctx().launches += NL;
}

}  // namespace

int mlp_param_count() { return param_count(); }

void mlp_forward(cudaStream_t s, const float *P, const float *norm, const float *X, int B, float *Y) {
    if (B <= 0) return;
    DBuf h1(sizeof(float) * (size_t)B * DIMS[1], s), h2(sizeof(float) * (size_t)B * DIMS[2], s);
    float *acts[NL] = {(float *)h1.get(), (float *)h2.get(), Y};
    forward(s, P, norm, X, B, acts);
}

// One training step on a batch: forward, loss, backward, Adam (lr > 0).  G receives the
// gradient (same layout as P); loss (device scalar) receives the batch loss.
void mlp_train_step(cudaStream_t s, float *P, float *M, float *V, const float *norm, const float *X, const float *T,
                    const float *reached, int B, float lr, int step, float *loss, float *G) {
    const int np = param_count();
    DBuf a1(sizeof(float) * (size_t)B * DIMS[1], s), a2(sizeof(float) * (size_t)B * DIMS[2], s),
        a3(sizeof(float) * (size_t)B * DIMS[3], s);
    DBuf d3(sizeof(float) * (size_t)B * DIMS[3], s), d2(sizeof(float) * (size_t)B * DIMS[2], s),
        d1(sizeof(float) * (size_t)B * DIMS[1], s);
    float *acts[NL] = {(float *)a1.get(), (float *)a2.get(), (float *)a3.get()};
    float *dacts[NL] = {(float *)d1.get(), (float *)d2.get(), (float *)d3.get()};
    forward(s, P, norm, X, B, acts);
    RSVD_CK(cudaMemsetAsync(loss, 0, sizeof(float), s));
    const int nout = B * DIMS[NL];
    mlp_loss_kernel<<<blocks_for(nout), 256, 0, s>>>(acts[NL - 1], T, reached, nout, 1.f / (float)nout, dacts[NL - 1],
                                                     loss);
    for (int l = NL - 1; l >= 0; l--) {
        const int in = DIMS[l], out = DIMS[l + 1];
        const float *W = P + w_off(l);
        float *dW = G + w_off(l), *db = dW + in * out;
        mlp_dz_kernel<<<blocks_for((long long)B * out), 256, 0, s>>>(dacts[l], acts[l], B * out, l < NL - 1);
        const float *Xin = (l == 0) ? X : acts[l - 1];
        mlp_dw_kernel<<<blocks_for((long long)in * out + out), 256, 0, s>>>(Xin, in, l == 0 ? norm : nullptr, dacts[l],
                                                                           out, B, dW, db);
        if (l > 0) mlp_dx_kernel<<<blocks_for((long long)B * in), 256, 0, s>>>(dacts[l], out, W, in, B, dacts[l - 1]);
    }
    if (lr > 0.f) {
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f / (1.f - powf(b1, (float)step)), c2 = 1.f / (1.f - powf(b2, (float)step));
        adam_kernel<<<blocks_for(np), 256, 0, s>>>(P, G, M, V, np, lr, b1, b2, 1e-8f, c1, c2);
    }
    RSVD_LAUNCH_CK();
    ctx().launches += 2 + 3 * NL;
}

void mlp_dims(int *d) {
    for (int l = 0; l <= NL; l++) d[l] = DIMS[l];
}

}  // namespace rsvd
