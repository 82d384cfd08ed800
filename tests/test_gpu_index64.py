"""librsvdpack64.so on the GPU: the int64_t-dimension API gives the results of the int API on
the same inputs, and takes a matrix of more than 2^31 entries (the case the reference's 64-bit
variant exists for, multi_core_mkl_code_64bit/README)."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import spectrum_matrix
from lowrankmatrixdecompositioncodes_gb300 import load_engine, load_engine64
from lowrankmatrixdecompositioncodes_gb300.capi import SeededOmega

pytestmark = pytest.mark.gpu


def _both():
    e32, e64 = load_engine(), load_engine64()
    for e in (e32, e64):
        e.set_precision("fp64")
        e.set_use_provider(True)
    return e32, e64


def _run(eng, fn, *args):
    eng.set_omega(SeededOmega(11))
    eng.lib.rsvdpack_reset_omega_counter()
    out = getattr(eng, fn)(*args)
    eng.check()
    return out


def test_fixed_rank_svd_matches_the_int_library():
    e32, e64 = _both()
    A = spectrum_matrix(700, 420, 0.93 ** np.arange(420), seed=5)
    U1, S1, V1 = _run(e32, "low_rank_svd_rand_decomp_fixed_rank", A, 40, 8, 1, 2, 1)
    U2, S2, V2 = _run(e64, "low_rank_svd_rand_decomp_fixed_rank", A, 40, 8, 1, 2, 1)
    assert U2.shape == (700, 40) and S2.shape == (40, 40) and V2.shape == (420, 40)
    np.testing.assert_allclose(np.diag(S2), np.diag(S1), rtol=1e-12, atol=0)
    # same factors up to the rounding of the products (column signs included)
    assert np.max(np.abs(U2 - U1)) < 1e-9 and np.max(np.abs(V2 - V1)) < 1e-9


def test_qb_id_cur_match_the_int_library():
    e32, e64 = _both()
    A = spectrum_matrix(600, 500, 0.9 ** np.arange(500), seed=8)
    Q1, B1, f1 = _run(e32, "randQB_pb_new", A, 16, 0, 1e-6 * np.linalg.norm(A), 1, 1)
    Q2, B2, f2 = _run(e64, "randQB_pb_new", A, 16, 0, 1e-6 * np.linalg.norm(A), 1, 1)
    assert f1 == f2 > 0 and Q2.shape == Q1.shape
    assert np.max(np.abs(Q2 @ B2 - Q1 @ B1)) < 1e-9 * np.linalg.norm(A)
    I1, T1 = _run(e32, "id_rand_decomp_fixed_rank", A, 30, 10, 2, 1)
    I2, T2 = _run(e64, "id_rand_decomp_fixed_rank", A, 30, 10, 2, 1)
    assert np.array_equal(I1, I2)
    np.testing.assert_allclose(T2, T1, rtol=0, atol=1e-9 * max(1.0, np.abs(T1).max()))
    C1, U1, R1 = _run(e32, "cur_rand_decomp_fixed_rank", A, 30, 10, 2, 1)
    C2, U2, R2 = _run(e64, "cur_rand_decomp_fixed_rank", A, 30, 10, 2, 1)
    assert np.array_equal(C1, C2) and np.array_equal(R1, R2)
    np.testing.assert_allclose(U2, U1, rtol=0, atol=1e-8 * np.abs(U1).max())


def _mem_available_gb():
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) / 2**20
    except OSError:
        pass
    return 0.0


def test_more_than_2_31_entries():
    """65536 x 32800 (2.15e9 entries, 17.2 GB of FP64) of rank 12, s_i = 2^-i: the fixed-rank
    rSVD through the 64-bit API recovers the singular values and the left singular vectors."""
    m, n, r = 65536, 32800, 12
    assert m * n > 2**31
    if _mem_available_gb() < 80:
        pytest.skip("needs about 40 GB of free host memory")
    g = np.random.default_rng(21)
    Ut, _ = np.linalg.qr(g.standard_normal((m, r)))
    Vt, _ = np.linalg.qr(g.standard_normal((n, r)))
    s = 2.0 ** -np.arange(r)
    A = ((Vt * s) @ Ut.T).T                # m x n, Fortran-ordered: no copy in to_mat
    assert A.flags.f_contiguous
    e64 = load_engine64()
    e64.set_precision("fp64")
    e64.set_use_provider(False)
    M = e64.to_mat(A)
    del A
    k, p = 8, 8
    U, S, V = e64.PMat(), e64.PMat(), e64.PMat()
    fr = C.c_int64(0)
    try:
        e64.lib.low_rank_svd_rand_decomp_fixed_rank(M, k, p, 1, 1, 1, C.byref(fr), C.byref(U), C.byref(S),
                                                    C.byref(V))
    finally:
        e64.lib.matrix_delete(M)
    e64.check()
    U, S, V = e64.from_mat(U), e64.from_mat(S), e64.from_mat(V)
    assert U.shape == (m, k) and V.shape == (n, k)
    np.testing.assert_allclose(np.diag(S), s[:k], rtol=1e-10)
    np.testing.assert_allclose(np.abs(np.sum(U * Ut[:, :k], axis=0)), 1.0, atol=1e-9)
    np.testing.assert_allclose(np.abs(np.sum(V * Vt[:, :k], axis=0)), 1.0, atol=1e-9)
