"""The learned rank / power-count proposal: training on the GPU through the engine's own MLP
kernels (rsvdpack_mlp_train_step / rsvdpack_mlp_forward, csrc/k_mlp.cu), the weights file,
and the decision rule.

Model: features (dataset.feature_vector: the probe's R-diagonal, the energy it leaves, log
sizes, log TOL) -> predicted log2(width / 32) of the single-shot range finder for q = 1 and q = 2.
A margin per output (the validation set's 60th percentile of target - prediction over runs
that reached the tolerance) is added before the width is used: an undersized proposal costs
one more block of the adaptive continuation, an oversized one costs columns in every block.

Weights file (little-endian): b"RSVDMLP1", int32 ndims, int32 dims[ndims], int32 nparams,
int32 nnorm, float32 params[nparams], float32 norm[nnorm], float32 margin[dims[-1]].
"""
from __future__ import annotations

import ctypes as C
import struct

import numpy as np

from . import dataset

MAGIC = b"RSVDMLP1"
QS = dataset.QS


def he_init(dims, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    parts = []
    for l in range(len(dims) - 1):
        i, j = dims[l], dims[l + 1]
        parts.append(rng.standard_normal(i * j) * np.sqrt(2.0 / i))
        parts.append(np.zeros(j))
    return np.concatenate(parts).astype(np.float32)


def targets(widths: np.ndarray) -> np.ndarray:
    return np.log2(np.asarray(widths, np.float64) / 32.0).astype(np.float32)


class Trainer:
    """Drives the engine's MLP kernels on device buffers (torch tensors as memory)."""

    def __init__(self, engine):
        import torch
        self.torch = torch
        self.L = engine.lib
        self.engine = engine
        L = self.L
        L.rsvdpack_mlp_train_step.argtypes = [C.c_void_p] * 7 + [C.c_int, C.c_float, C.c_int, C.c_void_p, C.c_void_p]
        L.rsvdpack_mlp_train_step.restype = C.c_int
        L.rsvdpack_mlp_forward.argtypes = [C.c_void_p] * 3 + [C.c_int, C.c_void_p]
        L.rsvdpack_mlp_forward.restype = C.c_int
        dims = (C.c_int * 4)()
        npar = C.c_int(0)
        if L.rsvdpack_mlp_info(dims, C.byref(npar)) != 0:
            raise RuntimeError(engine.last_error())
        self.dims = tuple(dims)
        self.nparams = npar.value

    def _dev(self, a):
        return self.torch.tensor(np.ascontiguousarray(a, np.float32), device="cuda")

    def predict(self, P, norm, X, batch=4096) -> np.ndarray:
        dP, dn = self._dev(P), self._dev(norm)
        out = []
        for i in range(0, len(X), batch):
            dX = self._dev(X[i:i + batch])
            dY = self.torch.empty(len(dX), self.dims[-1], device="cuda")
            if self.L.rsvdpack_mlp_forward(dP.data_ptr(), dn.data_ptr(), dX.data_ptr(), len(dX), dY.data_ptr()):
                raise RuntimeError(self.engine.last_error())
            out.append(dY.cpu().numpy())
        return np.concatenate(out)

    def fit(self, F, T, R, epochs=80, batch=256, lr=2e-3, seed=0, log=print):
        torch = self.torch
        rng = np.random.default_rng(seed)
        mean = F.mean(axis=0)
        std = F.std(axis=0) + 1e-6
        norm = np.concatenate([mean, 1.0 / std]).astype(np.float32)
        P = he_init(self.dims, seed)
        dP, dn = self._dev(P), self._dev(norm)
        dM, dV = torch.zeros_like(dP), torch.zeros_like(dP)
        dG = torch.empty_like(dP)
        dloss = torch.zeros(1, device="cuda")
        dF, dT, dR = self._dev(F), self._dev(T), self._dev(R)
        n = len(F)
        steps_total = epochs * ((n + batch - 1) // batch)
        step = 0
        for ep in range(epochs):
            perm = torch.tensor(rng.permutation(n), device="cuda")
            Fs, Ts, Rs = dF[perm].contiguous(), dT[perm].contiguous(), dR[perm].contiguous()
            tot = 0.0
            for i in range(0, n, batch):
                step += 1
                b = min(batch, n - i)
                lr_t = lr * 0.5 * (1.0 + np.cos(np.pi * step / steps_total))          # cosine decay
                rc = self.L.rsvdpack_mlp_train_step(dP.data_ptr(), dM.data_ptr(), dV.data_ptr(), dn.data_ptr(),
                                                    Fs[i:].data_ptr(), Ts[i:].data_ptr(), Rs[i:].data_ptr(), b,
                                                    C.c_float(lr_t), step, dloss.data_ptr(), dG.data_ptr())
                if rc:
                    raise RuntimeError(self.engine.last_error())
                tot += float(dloss.item()) * b
            if log and (ep % 10 == 0 or ep == epochs - 1):
                log(f"epoch {ep}: train loss {tot / n:.4f}")
        return dP.cpu().numpy(), norm


def calibrate_margin(pred: np.ndarray, T: np.ndarray, R: np.ndarray, quantile=0.6) -> np.ndarray:
    m = np.zeros(pred.shape[1], np.float32)
    for j in range(pred.shape[1]):
        ok = R[:, j] > 0
        m[j] = max(0.0, float(np.quantile(T[ok, j] - pred[ok, j], quantile))) if ok.any() else 0.0
    return m


def save(path: str, dims, P: np.ndarray, norm: np.ndarray, margin: np.ndarray) -> None:
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(struct.pack("<i", len(dims)))
        f.write(struct.pack(f"<{len(dims)}i", *dims))
        f.write(struct.pack("<ii", P.size, norm.size))
        f.write(np.asarray(P, "<f4").tobytes())
        f.write(np.asarray(norm, "<f4").tobytes())
        f.write(np.asarray(margin, "<f4").tobytes())


def load(path: str):
    with open(path, "rb") as f:
        if f.read(8) != MAGIC:
            raise ValueError("not an RSVDMLP1 weights file")
        nd = struct.unpack("<i", f.read(4))[0]
        dims = struct.unpack(f"<{nd}i", f.read(4 * nd))
        npar, nnorm = struct.unpack("<ii", f.read(8))
        P = np.frombuffer(f.read(4 * npar), "<f4").copy()
        norm = np.frombuffer(f.read(4 * nnorm), "<f4").copy()
        margin = np.frombuffer(f.read(4 * dims[-1]), "<f4").copy()
    return dims, P, norm, margin


def propose(pred_log2: np.ndarray, margin: np.ndarray, rmin: int) -> tuple[int, int]:
    """(width, q) from the network's outputs: widths 32 * 2^(pred + margin) rounded up to a
    multiple of 32 and capped at min(m, n); the q with the fewest passes x width (a pass of
    the single-shot method with q power iterations costs (2q + 2) products of that width)."""
    best = None
    for j, q in enumerate(QS):
        w = int(32 * np.ceil(2.0 ** (float(pred_log2[j]) + float(margin[j]))))
        w = max(32, min(rmin, w))
        cost = (2 * q + 2) * w
        if best is None or cost < best[0]:
            best = (cost, w, q)
    return best[1], best[2]
