"""Parity of the FP64X mode (FP64 data; large products FP64-accurate on the FP32 pipe by
double-float arithmetic; the l x l SVD as the FP32 Jacobi refined to FP64 accuracy), through the
C ABI, against the oracle on the same supplied test matrices.

* Every golden fixture of the reference's own build (tests/golden): singular values to 1e-10
  relative, sign-aligned factors to 1e-8, pivot / index sets exact -- the FP64 mode's bar.
* The plain fixed-rank workload at full size (2000 x 1000, s_i = 10^(-6(i-1)/999), k=100, p=10,
  q=2): the same bar against the oracle, and a residual equal to the oracle's.
* A two-sided ID / CUR at 8000 x 4000 (s_i = i^-2, k=200, p=20, q=2): index sets identical to
  the oracle's; T and S to 1e-6 of their largest entry; the CUR residual equal to the oracle's
  to 1e-6 relative (U itself solves a system of condition ~1e9, so it is compared to 1e-3).
"""
import numpy as np
import pytest

from conftest import golden_cases, load_golden, spectrum_matrix
from lowrankmatrixdecompositioncodes_gb300.capi import ListOmega, SeededOmega
from parity import compare_outputs

pytestmark = pytest.mark.gpu

GOLDEN_KEYS = sorted(golden_cases())


@pytest.fixture(autouse=True)
def fp64x_mode(engine):
    engine.set_precision("fp64x")
    engine.set_use_provider(True)
    yield
    engine.set_precision("fp64")


@pytest.mark.parametrize("key", GOLDEN_KEYS)
def test_fp64x_matches_reference_golden(engine, key):
    meta, A, want, omegas = load_golden(key)
    routine = meta["routine"]
    engine.set_omega(ListOmega(omegas))
    got = getattr(engine, routine)(A, *meta["args"])
    engine.check()
    got = got if isinstance(got, tuple) else (got,)
    compare_outputs(routine, got, want, rtol=1e-8)
    if routine in ("low_rank_svd_rand_decomp_fixed_rank", "low_rank_svd_blockrand_decomp_fixed_rank_or_prec"):
        s_got, s_want = np.diag(got[1]), np.diag(want[1])
        assert np.max(np.abs(s_got - s_want) / np.abs(s_want)) < 1e-10


def test_fp64x_plain_fixed_rank_workload_matches_oracle(engine, port):
    m, n = 2000, 1000
    s_all = 10.0 ** (-6.0 * np.arange(n) / (n - 1))
    A = spectrum_matrix(m, n, s_all, seed=2024)
    outs = []
    for lib in (port, engine):
        lib.set_omega(SeededOmega(99))
        outs.append(lib.low_rank_svd_rand_decomp_fixed_rank(A, 100, 10, 1, 2, 1))
    engine.check()
    (Uo, So, Vo), (Ue, Se, Ve) = outs
    so, se = np.diag(So), np.diag(Se)
    assert np.max(np.abs(se - so) / so) < 1e-10
    compare_outputs("low_rank_svd_rand_decomp_fixed_rank", (Ue, Se, Ve), (Uo, So, Vo), rtol=1e-8)
    res = np.linalg.norm(A - (Ue * se) @ Ve.T) / np.linalg.norm(A)
    res_o = np.linalg.norm(A - (Uo * so) @ Vo.T) / np.linalg.norm(A)
    assert abs(res - res_o) <= 1e-10 * res_o


def test_fp64x_two_sided_id_and_cur_index_sets(engine, port):
    m, n, k, p, q = 8000, 4000, 200, 20, 2
    A = spectrum_matrix(m, n, np.arange(1, n + 1, dtype=float) ** -2.0, seed=31)
    res = []
    for lib in (port, engine):
        lib.set_omega(SeededOmega(77))
        res.append(lib.id_two_sided_rand_decomp_fixed_rank(A, k, p, q, 1))
    engine.check()
    (Ic_o, Ir_o, T_o, S_o), (Ic_e, Ir_e, T_e, S_e) = res
    assert np.array_equal(Ic_e, Ic_o) and np.array_equal(Ir_e, Ir_o)
    for got, want in ((T_e, T_o), (S_e, S_o)):
        assert np.max(np.abs(got - want)) / np.max(np.abs(want)) < 1e-6
    cur = []
    for lib in (port, engine):
        lib.set_omega(SeededOmega(78))
        cur.append(lib.cur_rand_decomp_fixed_rank(A, k, p, q, 1))
    engine.check()
    (C_o, U_o, R_o), (C_e, U_e, R_e) = cur
    assert np.array_equal(C_e, C_o) and np.array_equal(R_e, R_o)
    # U solves (R R^T) U^T = R V, condition ~(s_1 / s_k)^2 = 1.6e9 here: the double-float products'
    # ~1e-14 is amplified to ~1e-5 in U, while the CUR residual agrees to many digits
    assert np.max(np.abs(U_e - U_o)) / np.max(np.abs(U_o)) < 1e-3
    fro = np.linalg.norm(A)
    res_e = np.linalg.norm(A - C_e @ U_e @ R_e) / fro
    res_o = np.linalg.norm(A - C_o @ U_o @ R_o) / fro
    assert abs(res_e - res_o) <= 1e-6 * res_o
