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
