"""Residual norms of a low-rank approximation on the device (rsvdpack_dev_residual_norms), through
the C ABI, against numpy in FP64: A = U diag(s) V^T with a known spectrum, approximated by its
leading k singular triplets (so the exact Frobenius residual is sqrt(sum_{i>k} s_i^2) and the
exact spectral residual is s_{k+1}) and by a perturbed version of them (residual checked against
numpy's norms of the formed residual).  FP64 and FP32 device data; a residual nine orders below
||A|| in FP64 keeps its digits.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _bind(L):
    L.rsvdpack_dev_residual_norms.restype = C.c_int
    L.rsvdpack_dev_residual_norms.argtypes = [C.c_void_p, C.c_int, C.c_longlong, C.c_int, C.c_int, C.c_void_p,
                                              C.c_longlong, C.c_void_p, C.c_void_p, C.c_longlong, C.c_int, C.c_int,
                                              C.POINTER(C.c_double), C.POINTER(C.c_double)]


def _dev(x, dt):
    return torch.from_numpy(np.ascontiguousarray(x.T)).to(dtype=dt, device="cuda")


def _norms(engine, A, U, S, V, dt, iters=30):
    L = engine.lib
    m, n = A.shape
    k = U.shape[1]
    dA, dU, dV = _dev(A, dt), _dev(U, dt), _dev(V, dt)
    dS = torch.from_numpy(S.copy()).cuda()
    fro, spec = C.c_double(0), C.c_double(0)
    rc = L.rsvdpack_dev_residual_norms(dA.data_ptr(), 0 if dt == torch.float64 else 1, m, m, n, dU.data_ptr(), m,
                                       dS.data_ptr(), dV.data_ptr(), n, k, iters, C.byref(fro), C.byref(spec))
    assert rc == 0, engine.last_error()
    return fro.value, spec.value


@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
def test_truncated_svd_residual_norms(engine, dt):
    _bind(engine.lib)
    g = np.random.default_rng(1)
    m, n, k = 3000, 1200, 60
    s = 0.93 ** np.arange(n)
    U, _ = np.linalg.qr(g.standard_normal((m, n)))
    V, _ = np.linalg.qr(g.standard_normal((n, n)))
    A = (U * s) @ V.T
    if dt == torch.float32:
        A = A.astype(np.float32).astype(np.float64)
    fro, spec = _norms(engine, A, U[:, :k], s[:k], V[:, :k], dt)
    want_fro = np.sqrt(np.sum(s[k:] ** 2))
    tol = 1e-9 if dt == torch.float64 else 1e-4
    assert abs(fro - want_fro) <= tol * want_fro + (0 if dt == torch.float64 else 1e-7 * np.linalg.norm(s))
    assert abs(spec - s[k]) <= 2e-3 * s[k]           # s_{k+1} / s_{k+2} = 1/0.93: converged


def test_small_residual_keeps_digits_in_fp64(engine):
    """||A - U S V^T|| ~ 1e-9 ||A||: the FP64 path forms the residual with FP64-accurate products."""
    _bind(engine.lib)
    g = np.random.default_rng(2)
    m, n, k = 2000, 800, 40
    s = np.concatenate([np.ones(k), 1e-9 * 0.5 ** np.arange(n - k)])
    U, _ = np.linalg.qr(g.standard_normal((m, n)))
    V, _ = np.linalg.qr(g.standard_normal((n, n)))
    A = (U * s) @ V.T
    Up = U[:, :k] + 1e-11 * g.standard_normal((m, k))
    R = A - (Up * s[:k]) @ V[:, :k].T
    fro, spec = _norms(engine, A, Up, s[:k], V[:, :k], torch.float64, iters=40)
    want_fro = np.linalg.norm(R)
    want_spec = np.linalg.norm(R, 2)
    assert abs(fro - want_fro) <= 2e-3 * want_fro
    assert want_spec * (1 - 1e-2) <= spec <= want_spec * (1 + 1e-6)
