"""FP64-accurate l x l steps of the mixed modes, through the C ABI.

* rsvdpack_dev_gemm_df64: FP64 products computed on the FP32 pipe in double-float arithmetic,
  against numpy's FP64 product (every transpose form, split-K and single-pass shapes): error
  within 1e-13 of |A||B| entrywise (FP64 itself gives ~1e-16 K).
* rsvdpack_dev_small_svd with fp32 == 2 (the mixed modes' l x l SVD: FP32 one-sided Jacobi,
  then the refinement): singular values within 1e-12 relative of the FP64 Jacobi
  (fp32 == 0) and of LAPACK on the same matrix, for a 272 x 272 upper-triangular factor whose
  spectrum has the shape of the 16384 x 8192 noisy workload's sketch (a dozen separated values
  above ~260 values packed into 27% of their range) and for well-separated spectra; factors
  orthonormal and reproducing the matrix to FP64 accuracy (to ~1e-10 where singular values lie
  closer than 1e-6 relative).
* A graded matrix (singular values over 8 decades): the refined values keep an absolute accuracy
  of order 1e-12 sigma_1 (the double-float products' error relative to |X||V|); the relative
  accuracy of the smallest ones is that divided by sigma_i / sigma_1 -- the FP64 Jacobi (fp32 == 0)
  is the form for strongly graded factors.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _bind(L):
    L.rsvdpack_dev_gemm_df64.restype = C.c_int
    L.rsvdpack_dev_gemm_df64.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_void_p,
                                         C.c_longlong, C.c_void_p, C.c_longlong, C.c_double, C.c_void_p,
                                         C.c_longlong]
    L.rsvdpack_dev_small_svd.restype = C.c_int
    L.rsvdpack_dev_small_svd.argtypes = [C.c_void_p, C.c_int, C.c_longlong, C.c_void_p, C.c_longlong, C.c_void_p,
                                         C.c_void_p, C.c_longlong, C.c_int]


def _dev(x):
    """numpy (rows x cols) -> column-major device tensor (its transpose, row-major)."""
    return torch.from_numpy(np.ascontiguousarray(x.T)).cuda()


@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
@pytest.mark.parametrize("M,N,K", [(272, 272, 272), (64, 48, 3000), (700, 130, 90), (1, 1, 1)])
def test_df64_gemm_matches_fp64(engine, ta, tb, M, N, K):
    L = engine.lib
    _bind(L)
    g = np.random.default_rng(M * 7 + N * 3 + K + 10 * ta + tb)
    A = g.standard_normal((K, M) if ta else (M, K)) * np.exp(g.standard_normal(1))
    B = g.standard_normal((N, K) if tb else (K, N))
    C0 = g.standard_normal((M, N))
    dA, dB, dC = _dev(A), _dev(B), _dev(C0)
    alpha, beta = 0.75, -0.5
    rc = L.rsvdpack_dev_gemm_df64(ta, tb, M, N, K, alpha, dA.data_ptr(), A.shape[0], dB.data_ptr(), B.shape[0],
                                  beta, dC.data_ptr(), M)
    assert rc == 0, engine.last_error()
    got = dC.cpu().numpy().T
    opA = A.T if ta else A
    opB = B.T if tb else B
    want = alpha * (opA @ opB) + beta * C0
    bound = 1e-13 * (np.abs(opA) @ np.abs(opB)) + 1e-15 * np.abs(C0)
    assert np.all(np.abs(got - want) <= bound + 1e-300)


def _spectrum(kind, n, g):
    if kind == "sketch":
        # a dozen separated values (i^-1.5), then ~260 values packed between 0.0166 and 0.0218
        head = np.arange(1, 14) ** -1.5
        tail = np.sort(0.0166 + 0.0052 * g.beta(1.3, 1.0, n - 13))[::-1]
        return np.concatenate([head, tail])
    if kind == "separated":
        return np.linspace(1.0, 0.05, n)
    if kind == "graded":
        return np.logspace(0, -8, n)
    raise ValueError(kind)


def _triangular_factor(s, g):
    n = len(s)
    Q1, _ = np.linalg.qr(g.standard_normal((n, n)))
    Q2, _ = np.linalg.qr(g.standard_normal((n, n)))
    X = (Q1 * s) @ Q2.T
    R = np.linalg.qr(X, mode="r")
    return R.T.copy()            # the engine runs its Jacobi on R^T


def _small_svd(engine, X, mode):
    L = engine.lib
    n = X.shape[0]
    G = _dev(X)
    U = torch.zeros(n, n, dtype=torch.float64, device="cuda")
    V = torch.zeros(n, n, dtype=torch.float64, device="cuda")
    S = torch.zeros(n, dtype=torch.float64, device="cuda")
    rc = L.rsvdpack_dev_small_svd(G.data_ptr(), n, n, U.data_ptr(), n, S.data_ptr(), V.data_ptr(), n, mode)
    assert rc >= 0, engine.last_error()
    return U.cpu().numpy().T, S.cpu().numpy(), V.cpu().numpy().T


@pytest.mark.parametrize("kind,n", [("sketch", 272), ("separated", 272), ("separated", 110), ("sketch", 96)])
def test_refined_small_svd_matches_fp64_jacobi(engine, kind, n):
    _bind(engine.lib)
    g = np.random.default_rng(n + len(kind))
    X = _triangular_factor(_spectrum(kind, n, g), g)
    U2, S2, V2 = _small_svd(engine, X, 2)
    _, S0, _ = _small_svd(engine, X, 0)
    S_lapack = np.linalg.svd(X, compute_uv=False)
    assert np.max(np.abs(S2 - S0) / S0) < 1e-12
    assert np.max(np.abs(S2 - S_lapack) / S_lapack) < 1e-12
    assert np.all(np.diff(S2) <= 0)
    I = np.eye(n)
    # the sketch-like spectrum has pairs closer than 1e-6 relative: the last first-order step
    # leaves their vectors orthogonal to ~|C|^2 ~ 1e-10 (singular values are second order in it)
    orth = 1e-9 if kind == "sketch" else 1e-12
    assert np.max(np.abs(U2.T @ U2 - I)) < orth
    assert np.max(np.abs(V2.T @ V2 - I)) < orth
    recon = np.linalg.norm(X - (U2 * S2) @ V2.T) / np.linalg.norm(X)
    assert recon < (1e-9 if kind == "sketch" else 1e-13), recon


def test_refined_small_svd_graded_absolute_accuracy(engine):
    _bind(engine.lib)
    g = np.random.default_rng(3)
    n = 128
    X = _triangular_factor(_spectrum("graded", n, g), g)
    _, S2, _ = _small_svd(engine, X, 2)
    S_lapack = np.linalg.svd(X, compute_uv=False)
    assert np.max(np.abs(S2 - S_lapack)) < 1e-11 * S_lapack[0]
