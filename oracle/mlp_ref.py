"""CPU oracle for the learned proposal's network (test infrastructure only: tests/ import
it to check the engine's CUDA kernels in csrc/k_mlp.cu; nothing on the product path does).

A plain float64 restatement of the same MLP: layers 36 -> 64 -> 64 -> 2, ReLU on the hidden
layers, inputs normalised by norm = [mean, inv_std]; parameters in one flat array, layer by
layer W_l (in x out, row-major) then b_l.  Loss per output: (y - t)^2 if the training run
reached the tolerance, max(0, t - y)^2 if not, averaged over batch x outputs.  Adam as in
Kingma & Ba (2015) with bias correction.  The reference project has no learned component;
this oracle is pinned by finite differences (tests/test_mlp.py).
"""
from __future__ import annotations

import numpy as np

DIMS = (36, 64, 64, 2)


def n_params(dims=DIMS) -> int:
    return sum(dims[l] * dims[l + 1] + dims[l + 1] for l in range(len(dims) - 1))


def unpack(P: np.ndarray, dims=DIMS):
    out, o = [], 0
    for l in range(len(dims) - 1):
        i, j = dims[l], dims[l + 1]
        W = P[o:o + i * j].reshape(i, j)
        o += i * j
        b = P[o:o + j]
        o += j
        out.append((W, b))
    return out


def forward(P, norm, X, dims=DIMS):
    """Returns the list of post-activation outputs of every layer (last = prediction)."""
    d0 = dims[0]
    h = (np.asarray(X, np.float64) - norm[:d0]) * norm[d0:2 * d0]
    acts = [h]
    layers = unpack(np.asarray(P, np.float64), dims)
    for l, (W, b) in enumerate(layers):
        z = h @ W + b
        h = np.maximum(z, 0.0) if l < len(layers) - 1 else z
        acts.append(h)
    return acts


def loss_and_grad(P, norm, X, T, reached, dims=DIMS):
    acts = forward(P, norm, X, dims)
    Y = acts[-1]
    d = Y - T
    d = np.where((reached == 0) & (d > 0), 0.0, d)
    cnt = d.size
    loss = float(np.sum(d * d) / cnt)
    dY = 2.0 * d / cnt
    layers = unpack(np.asarray(P, np.float64), dims)
    grads = [None] * len(layers)
    g = dY
    for l in range(len(layers) - 1, -1, -1):
        W, b = layers[l]
        if l < len(layers) - 1:
            g = g * (acts[l + 1] > 0)
        grads[l] = (acts[l].T @ g, g.sum(axis=0))
        g = g @ W.T
    G = np.concatenate([np.concatenate([dW.ravel(), db]) for dW, db in grads])
    return loss, G


def adam(P, G, M, V, lr, step, b1=0.9, b2=0.999, eps=1e-8):
    M = b1 * M + (1 - b1) * G
    V = b2 * V + (1 - b2) * G * G
    mh = M / (1 - b1 ** step)
    vh = V / (1 - b2 ** step)
    return P - lr * mh / (np.sqrt(vh) + eps), M, V


def init_params(seed: int, dims=DIMS) -> np.ndarray:
    """He-normal weights, zero biases (the training script's initialisation)."""
    rng = np.random.default_rng(seed)
    parts = []
    for l in range(len(dims) - 1):
        i, j = dims[l], dims[l + 1]
        parts.append(rng.standard_normal(i * j) * np.sqrt(2.0 / i))
        parts.append(np.zeros(j))
    return np.concatenate(parts)
