"""The learned proposal's network: the CPU oracle pinned by finite differences, and the
engine's CUDA forward / backward / Adam kernels (csrc/k_mlp.cu) checked against it on the
same parameters and batch."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import mlp_ref  # noqa: E402


def _batch(seed, B=48):
    g = np.random.default_rng(seed)
    X = g.standard_normal((B, mlp_ref.DIMS[0])) * 2.0 + 0.5
    T = g.standard_normal((B, mlp_ref.DIMS[-1])) + 3.0
    reached = (g.random((B, mlp_ref.DIMS[-1])) > 0.2).astype(np.float64)
    norm = np.concatenate([g.standard_normal(mlp_ref.DIMS[0]) * 0.1, 1.0 / (1.5 + g.random(mlp_ref.DIMS[0]))])
    return X, T, reached, norm


def test_oracle_gradient_matches_finite_differences():
    X, T, reached, norm = _batch(1)
    P = mlp_ref.init_params(3)
    _, G = mlp_ref.loss_and_grad(P, norm, X, T, reached)
    g = np.random.default_rng(5)
    idx = g.choice(P.size, 60, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros_like(P)
        e[i] = h
        lp, _ = mlp_ref.loss_and_grad(P + e, norm, X, T, reached)
        lm, _ = mlp_ref.loss_and_grad(P - e, norm, X, T, reached)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - G[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, G[i])


def test_oracle_adam_reduces_loss():
    X, T, reached, norm = _batch(2, B=128)
    P = mlp_ref.init_params(4)
    M = np.zeros_like(P)
    V = np.zeros_like(P)
    l0, _ = mlp_ref.loss_and_grad(P, norm, X, T, reached)
    for step in range(1, 201):
        _, G = mlp_ref.loss_and_grad(P, norm, X, T, reached)
        P, M, V = mlp_ref.adam(P, G, M, V, 3e-3, step)
    l1, _ = mlp_ref.loss_and_grad(P, norm, X, T, reached)
    assert l1 < 0.2 * l0


@pytest.mark.gpu
def test_gpu_kernels_match_the_oracle(engine):
    torch = pytest.importorskip("torch")
    L = engine.lib
    L.rsvdpack_mlp_train_step.argtypes = [C.c_void_p] * 7 + [C.c_int, C.c_float, C.c_int, C.c_void_p, C.c_void_p]
    L.rsvdpack_mlp_forward.argtypes = [C.c_void_p] * 3 + [C.c_int, C.c_void_p]
    dims = (C.c_int * 4)()
    npar = C.c_int(0)
    assert L.rsvdpack_mlp_info(dims, C.byref(npar)) == 0
    assert tuple(dims) == mlp_ref.DIMS and npar.value == mlp_ref.n_params()
    X, T, reached, norm = _batch(7, B=200)
    P = mlp_ref.init_params(11)
    f32 = lambda a: torch.tensor(np.asarray(a, np.float32), device="cuda")
    dP, dnorm, dX, dT, dR = f32(P), f32(norm), f32(X), f32(T), f32(reached)
    dM, dV = torch.zeros_like(dP), torch.zeros_like(dP)
    dG = torch.empty_like(dP)
    dloss = torch.zeros(1, device="cuda")
    # the oracle evaluated on the FP32-rounded inputs
    P32, n32, X32 = (np.asarray(a, np.float32).astype(np.float64) for a in (P, norm, X))
    T32 = np.asarray(T, np.float32).astype(np.float64)
    # forward
    dY = torch.empty(200, mlp_ref.DIMS[-1], device="cuda")
    torch.cuda.synchronize()
    assert L.rsvdpack_mlp_forward(dP.data_ptr(), dnorm.data_ptr(), dX.data_ptr(), 200, dY.data_ptr()) == 0
    Yo = mlp_ref.forward(P32, n32, X32)[-1]
    assert np.max(np.abs(dY.cpu().numpy() - Yo)) <= 1e-4 * (1 + np.max(np.abs(Yo)))
    # gradient (lr = 0: no update)
    assert L.rsvdpack_mlp_train_step(dP.data_ptr(), 0, 0, dnorm.data_ptr(), dX.data_ptr(), dT.data_ptr(),
                                     dR.data_ptr(), 200, C.c_float(0.0), 1, dloss.data_ptr(), dG.data_ptr()) == 0
    lo, Go = mlp_ref.loss_and_grad(P32, n32, X32, T32, reached)
    G = dG.cpu().numpy()
    assert abs(float(dloss.item()) - lo) <= 1e-4 * lo
    assert np.max(np.abs(G - Go)) <= 1e-4 * np.max(np.abs(Go)), np.max(np.abs(G - Go))
    # one Adam step
    assert L.rsvdpack_mlp_train_step(dP.data_ptr(), dM.data_ptr(), dV.data_ptr(), dnorm.data_ptr(), dX.data_ptr(),
                                     dT.data_ptr(), dR.data_ptr(), 200, C.c_float(1e-3), 1, dloss.data_ptr(),
                                     dG.data_ptr()) == 0
    Pn, _, _ = mlp_ref.adam(P32, Go, np.zeros_like(P32), np.zeros_like(P32), 1e-3, 1)
    assert np.max(np.abs(dP.cpu().numpy() - Pn)) <= 2e-5
