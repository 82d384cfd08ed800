"""The l x l kernels on their own (Cholesky, one-sided Jacobi SVD) against numpy, in both
compute types, across the sizes that select their different implementations (packed
shared memory / blocked / cluster / global-memory paths)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _bind(L):
    L.rsvdpack_dev_small_svd.restype = C.c_int
    L.rsvdpack_dev_small_svd.argtypes = [C.c_void_p, C.c_int, C.c_longlong, C.c_void_p, C.c_longlong, C.c_void_p,
                                         C.c_void_p, C.c_longlong, C.c_int]
    L.rsvdpack_dev_small_cholesky.restype = C.c_int
    L.rsvdpack_dev_small_cholesky.argtypes = [C.c_void_p, C.c_int, C.c_longlong, C.c_int]


def _dev(A):
    """column-major float64 device copy with ld = rows"""
    return torch.from_numpy(np.asfortranarray(A).T.copy()).cuda()


@pytest.mark.parametrize("fp32", [0, 1])
@pytest.mark.parametrize("n", [5, 33, 64, 110, 192, 200, 272, 288, 300, 400, 600])
def test_small_cholesky(engine, n, fp32):
    _bind(engine.lib)
    g = np.random.default_rng(n)
    X = g.standard_normal((n + 20, n))
    G = X.T @ X
    d = _dev(G)
    torch.cuda.synchronize()
    rc = engine.lib.rsvdpack_dev_small_cholesky(d.data_ptr(), n, n, fp32)
    assert rc == 0, engine.last_error()
    R = d.cpu().numpy().T
    assert np.allclose(np.tril(R, -1), 0)
    ref = np.linalg.cholesky(G).T
    tol = 2e-4 if fp32 else 1e-10
    assert np.max(np.abs(R - ref)) / np.max(np.abs(ref)) < tol


def test_small_cholesky_reports_breakdown(engine):
    _bind(engine.lib)
    n = 40
    X = np.random.default_rng(1).standard_normal((n, 10))
    G = X @ X.T                      # rank 10 < 40: not positive definite
    d = _dev(G)
    torch.cuda.synchronize()
    assert engine.lib.rsvdpack_dev_small_cholesky(d.data_ptr(), n, n, 0) == 4


# 97, 110, 112: the 8-CTA register-Gram form (block width 7) and its edges; 257, 272, 288: the
# 16-CTA one (block width 9) -- 257 leaves a whole padding block -- ; the others the one-sided form.
# fp32 = 2: the FP32 Jacobi refined to FP64 accuracy
@pytest.mark.parametrize("fp32", [0, 1, 2])
@pytest.mark.parametrize("n", [7, 40, 64, 97, 110, 112, 200, 257, 272, 288, 300, 400])
def test_small_svd(engine, n, fp32):
    _bind(engine.lib)
    g = np.random.default_rng(100 + n)
    # the refined form (fp32 == 2) on spectra spanning ~6 decades, its domain: below ~1e-8 sigma_1
    # the FP32 start carries no information (the FP64 mode takes the FP64 Jacobi there)
    s_true = 0.93 ** (np.arange(n) * (200 / n if fp32 == 2 and n > 200 else 1.0))
    Q1, _ = np.linalg.qr(g.standard_normal((n, n)))
    Q2, _ = np.linalg.qr(g.standard_normal((n, n)))
    A = (Q1 * s_true) @ Q2.T
    d = _dev(A)
    U = torch.zeros(n, n, dtype=torch.float64, device="cuda")
    V = torch.zeros(n, n, dtype=torch.float64, device="cuda")
    S = torch.zeros(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    sweeps = engine.lib.rsvdpack_dev_small_svd(d.data_ptr(), n, n, U.data_ptr(), n, S.data_ptr(), V.data_ptr(), n,
                                               fp32)
    assert sweeps > 0, engine.last_error()
    Uh, Sh, Vh = U.cpu().numpy().T, S.cpu().numpy(), V.cpu().numpy().T
    tol = 5e-5 if fp32 == 1 else 1e-12
    assert np.all(np.diff(Sh) <= 0)
    assert np.max(np.abs(Sh - s_true)) < tol
    assert np.max(np.abs(Uh @ np.diag(Sh) @ Vh.T - A)) < 10 * tol
    # the refined form keeps an absolute accuracy of ~1e-14 sigma_1, so the vectors of values far
    # below sigma_1 (here down to 0.93^399) are checked where sigma > 1e-3 sigma_1
    lead = np.arange(n) if fp32 != 2 else np.nonzero(s_true > 1e-3)[0]
    assert np.max(np.abs(Vh[:, lead].T @ Vh[:, lead] - np.eye(len(lead)))) < 10 * tol
