"""GPU checks of the host-facing helpers that run on the device: the GEMM wrappers
(matrix_matrix_mult and its transposed forms, MVF:538-561), the product formers and the
approximation reports (MVF:1304-1336, RRA:2337-2573), and the thin entry points over the validated
routines (randomized_low_rank_svd1..4, pivoted_QR_of_specified_rank), against numpy and the oracle.
FP64 mode."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import spectrum_matrix
from lowrankmatrixdecompositioncodes_gb300.capi import SeededOmega
from parity import compare_outputs

pytestmark = pytest.mark.gpu

libc = C.CDLL(None)


@pytest.fixture(autouse=True)
def fp64(engine):
    engine.set_precision("fp64")
    engine.set_use_provider(True)
    yield


def _mm(engine, name, A, B, shape):
    L = engine.lib
    getattr(L, name).argtypes = [engine.PMat] * 3
    MA, MB, MC = engine.to_mat(A), engine.to_mat(B), L.matrix_new(*shape)
    getattr(L, name)(MA, MB, MC)
    engine.check()
    L.matrix_delete(MA)
    L.matrix_delete(MB)
    return engine.from_mat(MC)


def test_gemm_wrappers(engine):
    g = np.random.default_rng(3)
    A, B = g.standard_normal((70, 50)), g.standard_normal((50, 33))
    np.testing.assert_allclose(_mm(engine, "matrix_matrix_mult", A, B, (70, 33)), A @ B, rtol=0, atol=1e-12)
    At = g.standard_normal((50, 70))
    np.testing.assert_allclose(_mm(engine, "matrix_transpose_matrix_mult", At, B, (70, 33)), At.T @ B, rtol=0,
                               atol=1e-12)
    Bt = g.standard_normal((33, 50))
    np.testing.assert_allclose(_mm(engine, "matrix_matrix_transpose_mult", A, Bt, (70, 33)), A @ Bt.T, rtol=0,
                               atol=1e-12)


def test_product_formers_and_reports(engine, capfd):
    L = engine.lib
    g = np.random.default_rng(4)
    U, V = np.linalg.qr(g.standard_normal((60, 8)))[0], np.linalg.qr(g.standard_normal((40, 8)))[0]
    S = np.diag(np.linspace(3, 1, 8))
    for name in ("form_svd_product_matrix", "form_cur_product_matrix"):
        getattr(L, name).argtypes = [engine.PMat] * 4
    MU, MS, MV, P = engine.to_mat(U), engine.to_mat(S), engine.to_mat(V), L.matrix_new(60, 40)
    L.form_svd_product_matrix(MU, MS, MV, P)
    engine.check()
    np.testing.assert_allclose(engine.from_mat(P), U @ S @ V.T, rtol=0, atol=1e-12)
    Cm, Um, Rm = g.standard_normal((60, 5)), g.standard_normal((5, 5)), g.standard_normal((5, 40))
    MC, MUc, MR, P = engine.to_mat(Cm), engine.to_mat(Um), engine.to_mat(Rm), L.matrix_new(60, 40)
    L.form_cur_product_matrix(MC, MUc, MR, P)
    engine.check()
    np.testing.assert_allclose(engine.from_mat(P), Cm @ Um @ Rm, rtol=0, atol=1e-12)
    A = U @ S @ V.T + 1e-3 * g.standard_normal((60, 40))
    MA = engine.to_mat(A)
    L.use_low_rank_svd_for_approximation.argtypes = [engine.PMat] * 4
    capfd.readouterr()
    L.use_low_rank_svd_for_approximation(MA, MU, MS, MV)
    libc.fflush(None)
    out = capfd.readouterr().out
    got = float(re.search(r"percent error = ([0-9.eE+-]+)", out).group(1))
    want = 100 * np.linalg.norm(A - U @ S @ V.T) / np.linalg.norm(A)
    assert abs(got - want) < 1e-5 * want
    for x in (MU, MS, MV, MC, MUc, MR, MA):
        L.matrix_delete(x)


def test_older_entry_points_and_rank_only_qr_match_the_oracle(engine, port):
    L = engine.lib
    for name, n_int in (("randomized_low_rank_svd2", 1), ("randomized_low_rank_svd3", 3),
                        ("randomized_low_rank_svd4", 3)):
        getattr(L, name).argtypes = [engine.PMat] + [engine.Int] * n_int + [C.POINTER(engine.PMat)] * 3
    A = spectrum_matrix(150, 100, 0.9 ** np.arange(100), seed=6)

    def old(name, *a):
        engine.set_omega(SeededOmega(5))
        M = engine.to_mat(A)
        U, S, V = engine.PMat(), engine.PMat(), engine.PMat()
        getattr(L, name)(M, *a, C.byref(U), C.byref(S), C.byref(V))
        engine.check()
        L.matrix_delete(M)
        return engine.from_mat(U), engine.from_mat(S), engine.from_mat(V)

    for name, a_old, a_new in (("randomized_low_rank_svd2", (12,), (12, 0, 1, 1, 1)),
                               ("randomized_low_rank_svd3", (12, 3, 1), (12, 0, 1, 3, 1))):
        port.set_omega(SeededOmega(5))
        want = port.low_rank_svd_rand_decomp_fixed_rank(A, *a_new)
        compare_outputs("low_rank_svd_rand_decomp_fixed_rank", old(name, *a_old), want, rtol=1e-8)
    U4, S4, V4 = old("randomized_low_rank_svd4", 8, 3, 1)
    assert U4.shape == (150, 24) and np.all(np.diff(np.diag(S4)) >= 0)           # ascending
    port.set_omega(SeededOmega(5))
    Q, B = port.randQB_pb(A, 8, 3, 1, 1)
    Up, Sp, Vp = port.low_rank_svd_rand_decomp_fromQB(Q, B)
    top = slice(24 - 12, 24)                  # the well-resolved half of the 24 pairs
    np.testing.assert_allclose(np.diag(S4)[top], np.diag(Sp)[::-1][top], rtol=1e-9)
    got = engine.pivoted_QR_of_specified_rank(A, 20)
    want = port.pivoted_QR_of_specified_rank(A, 20)
    compare_outputs("pivoted_QR_of_specified_rank", got, want, rtol=1e-8)
