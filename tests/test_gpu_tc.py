"""Tensor-core (tcgen05) products and the mixed-precision rSVD path, through the C ABI.

Products are checked against an FP64 product of the same operands: TF32 operands keep
10 mantissa bits, BF16 operands 7, both accumulate in FP32, so the error relative to
the result's scale is bounded by ~2^-10 (TF32) / ~2^-7 (BF16) times a small factor.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import spectrum_matrix
from lowrankmatrixdecompositioncodes_gb300.capi import SeededOmega

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = {"tf32": 3e-3, "bf16": 2e-2}


def _bind(L):
    L.rsvdpack_dev_sketch.restype = C.c_int
    L.rsvdpack_dev_sketch.argtypes = [C.c_void_p, C.c_int, C.c_longlong, C.c_int, C.c_int, C.c_void_p,
                                      C.c_longlong, C.c_int, C.c_void_p, C.c_longlong, C.c_int]


def colmajor(rows, cols, ld, gen):
    """A column-major rows x cols float32 matrix on the GPU with leading dimension ld."""
    buf = torch.zeros(cols, ld, device="cuda", dtype=torch.float32)
    buf[:, :rows] = torch.randn(cols, rows, device="cuda", generator=gen)
    return buf


def view(buf, rows):
    return buf[:, :rows].T.double()


@pytest.mark.parametrize("prec", ["tf32", "bf16"])
@pytest.mark.parametrize("trans", [1, 0])
@pytest.mark.parametrize("m,n,w", [(300, 500, 40), (1000, 777, 272), (4100, 2048, 130), (520, 1030, 600),
                                   (2000, 1000, 110), (128, 64, 16)])
def test_tc_product_matches_fp64(engine, prec, trans, m, n, w):
    _bind(engine.lib)
    engine.set_precision(prec)
    g = torch.Generator(device="cuda")
    g.manual_seed(m * 31 + n * 7 + w + trans)
    lda = (m + 31) // 32 * 32
    A = colmajor(m, n, lda, g)
    xr, yr = (m, n) if trans else (n, m)
    ldx, ldy = (xr + 31) // 32 * 32, (yr + 31) // 32 * 32
    X = colmajor(xr, w, ldx, g)
    Y = torch.full((w, ldy), float("nan"), device="cuda", dtype=torch.float32)
    torch.cuda.synchronize()
    rc = engine.lib.rsvdpack_dev_sketch(A.data_ptr(), 1, lda, m, n, X.data_ptr(), ldx, w, Y.data_ptr(), ldy, trans)
    assert rc == 0, engine.last_error()
    t = engine.last_timing()
    Ad, Xd = view(A, m), view(X, xr)
    ref = (Ad.T @ Xd) if trans else (Ad @ Xd)
    got = view(Y, yr)
    err = float((got - ref).abs().max() / ref.abs().max())
    # A X (MN-major A operand) always runs kind::f16 on bf16 operands; A^T X runs
    # kind::tf32 in TF32 mode
    kind = "tf32" if (prec == "tf32" and trans == 1) else "bf16"
    assert err < TOL[kind], f"relative error {err:.3e}"
    if m * n * w >= 4.0e6:   # smaller products go to the CUDA-core GEMM by design
        assert t.gemm_launches >= 1, "the tensor-core product did not run"
    # padding rows of Y beyond the product are untouched
    if ldy > yr:
        assert torch.isnan(Y[:, yr:]).all()
    engine.set_precision("fp64")


@pytest.mark.parametrize("prec,k,p", [("tf32", 64, 8), ("bf16", 64, 8), ("fp32", 300, 20), ("tf32", 300, 20)])
def test_mixed_precision_rsvd_matches_fp64_error(engine, prec, k, p):
    """Same method, same test matrix: the tensor-core path's relative Frobenius residual
    is within 1e-3 (relative) of the FP64 path's.  l = 320 exceeds the one-CTA Cholesky
    (order 288 in FP32) and runs the tiled global-memory factorisation."""
    m, n = 3000, 1500
    s = (1.0 + np.arange(n)) ** -1.5
    A = spectrum_matrix(m, n, s, seed=8) + 1e-4 * np.random.default_rng(9).standard_normal((m, n))
    res = {}
    for mode in ("fp64", prec):
        engine.set_precision(mode)
        engine.set_omega(SeededOmega(17))
        U, S, V = engine.low_rank_svd_rand_decomp_fixed_rank(A, k, p, 1, 2, 1)
        engine.check()
        res[mode] = np.linalg.norm(A - U @ S @ V.T) / np.linalg.norm(A)
    engine.set_precision("fp64")
    assert res[prec] <= res["fp64"] * (1 + 1e-3), res


def _bind3(L):
    L.rsvdpack_dev_gemm_3xtf32.restype = C.c_int
    L.rsvdpack_dev_gemm_3xtf32.argtypes = [C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong, C.c_int, C.c_int,
                                           C.c_int, C.c_void_p, C.c_longlong]
    L.rsvdpack_dev_update_3xtf32.restype = C.c_int
    L.rsvdpack_dev_update_3xtf32.argtypes = [C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong, C.c_int, C.c_int,
                                             C.c_int, C.c_void_p, C.c_longlong, C.POINTER(C.c_double)]


@pytest.mark.parametrize("M,N,K", [(1000, 300, 4096), (333, 130, 20000), (2048, 64, 777), (130, 520, 33)])
def test_3xtf32_product_is_fp32_accurate(engine, M, N, K):
    """D = A^T X from split operands: the error stays at FP32 level (~1e-6 of the product's
    scale) even for long K, where one FP32-accumulated tensor-core chain would drift."""
    _bind3(engine.lib)
    g = torch.Generator(device="cuda")
    g.manual_seed(M + N + K)
    lda, ldx, ldd = (K + 3) // 4 * 4, (K + 3) // 4 * 4, (M + 3) // 4 * 4
    A = colmajor(K, M, lda, g)
    X = colmajor(K, N, ldx, g)
    D = torch.full((N, ldd), float("nan"), device="cuda")
    torch.cuda.synchronize()
    rc = engine.lib.rsvdpack_dev_gemm_3xtf32(A.data_ptr(), lda, X.data_ptr(), ldx, M, N, K, D.data_ptr(), ldd)
    assert rc == 0, engine.last_error()
    ref = view(A, K).T @ view(X, K)
    err = float((view(D, M) - ref).norm() / ref.norm())
    assert err < 3e-6, err
    if ldd > M:
        assert torch.isnan(D[:, M:]).all()


# (M, N, K, ldc pad): N > 512 tiles by 256 columns, N <= 256 is one tile with a ragged last
# 64-column chunk (both through the TMA epilogue); 256 < N <= 512 is two MMA chunks, and an
# odd ldc or M % 4 != 0 (padding rows right after row M) take the register epilogue; M not
# a multiple of 128 leaves a ragged last row tile
@pytest.mark.parametrize("M,N,K,pad", [(1000, 700, 96, 4), (300, 200, 64, 0), (257, 530, 40, 3), (300, 400, 50, 4),
                                       (129, 1030, 288, 1), (4096, 2048, 256, 0), (260, 530, 40, 4),
                                       (1000, 130, 33, 8)])
def test_3xtf32_update_in_place(engine, M, N, K, pad):
    """C -= A^T X in one pass (the blocked-QB deflation): C close to A^T X, so the result is
    small against the terms; it must match FP64 to ~1e-6 of the terms' scale, leave padding
    rows untouched, and report ||C||_F^2 of the result."""
    _bind3(engine.lib)
    g = torch.Generator(device="cuda")
    g.manual_seed(M * 3 + N + K)
    lda, ldx = (K + 3) // 4 * 4, (K + 3) // 4 * 4
    ldc = M + pad if pad else M
    A = colmajor(K, M, lda, g)
    X = colmajor(K, N, ldx, g)
    prod = view(A, K).T @ view(X, K)
    Cm = torch.full((N, ldc), float("nan"), device="cuda")
    small = 1e-3 * torch.randn(N, M, device="cuda", generator=g, dtype=torch.float64)
    Cm[:, :M] = (prod.T + small).float()
    C0 = view(Cm, M).clone()
    fro2 = C.c_double(0.0)
    torch.cuda.synchronize()
    rc = engine.lib.rsvdpack_dev_update_3xtf32(A.data_ptr(), lda, X.data_ptr(), ldx, M, N, K, Cm.data_ptr(), ldc,
                                               C.byref(fro2))
    assert rc == 0, engine.last_error()
    ref = C0 - prod
    got = view(Cm, M)
    err = float((got - ref).norm() / prod.norm())
    assert err < 2e-6, err
    assert abs(fro2.value - float((got * got).sum())) <= 1e-5 * float((got * got).sum())
    if ldc > M:
        assert torch.isnan(Cm[:, M:]).all()
