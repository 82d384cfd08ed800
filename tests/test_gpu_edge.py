"""Edge cases through the C ABI, FP64 mode, engine against the oracle on the same supplied
test matrices: ragged shapes (no dimension a multiple of the engine's 32-element padding),
the largest sketch the reference allows (k + p = min(m, n)), single-column extremes, an
all-zero matrix and rank-deficient inputs (CholeskyQR breaks down there and the Householder
fallback must take over).  Singular values to 1e-10 of the largest, sign-aligned factors to
1e-8, index sets exactly."""
import numpy as np
import pytest

from conftest import spectrum_matrix
from lowrankmatrixdecompositioncodes_gb300.capi import SeededOmega
from parity import compare_outputs

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def fp64_mode(engine):
    engine.set_precision("fp64")
    engine.set_use_provider(True)
    yield


def _both(engine, port, routine, A, *args, seed=11):
    outs = []
    for lib in (port, engine):
        lib.set_omega(SeededOmega(seed))
        outs.append(getattr(lib, routine)(A, *args))
    engine.check()
    return outs


def _svals_close(got, want):
    s_got, s_want = np.diag(got[1]), np.diag(want[1])
    scale = max(np.max(np.abs(s_want)), 1e-300)
    assert np.max(np.abs(s_got - s_want)) <= 1e-10 * scale


@pytest.mark.parametrize("m,n,k,p", [(37, 23, 5, 3), (33, 97, 7, 4), (200, 20, 18, 2), (129, 65, 64, 1),
                                     (50, 1, 1, 0), (1, 40, 1, 0)])
def test_fixed_rank_ragged_and_maximal(engine, port, m, n, k, p):
    # 0.9^i keeps every compared singular vector well conditioned (sigma_k / sigma_1 >= 1e-3):
    # vectors of singular values near eps * sigma_1 are determined only to eps sigma_1 / sigma_j
    A = spectrum_matrix(m, n, 0.9 ** np.arange(min(m, n)), seed=m * 7 + n)
    want, got = _both(engine, port, "low_rank_svd_rand_decomp_fixed_rank", A, k, p, 1, 2, 1)
    _svals_close(got, want)
    compare_outputs("low_rank_svd_rand_decomp_fixed_rank", got, want, rtol=1e-8)


@pytest.mark.parametrize("m,n", [(45, 31), (31, 45)])
def test_id_and_cur_ragged(engine, port, m, n):
    A = spectrum_matrix(m, n, 0.6 ** np.arange(min(m, n)), seed=m + 3 * n)
    for routine, args in (("id_rand_decomp_fixed_rank", (9, 3, 2, 1)),
                          ("id_two_sided_rand_decomp_fixed_rank", (9, 3, 2, 1)),
                          ("cur_rand_decomp_fixed_rank", (9, 3, 2, 1)),
                          ("id_decomp_fixed_rank_or_prec", (8, 0.0))):
        want, got = _both(engine, port, routine, A, *args)
        compare_outputs(routine, got, want, rtol=1e-8)


def test_qb_tolerance_mode_ragged(engine, port):
    A = spectrum_matrix(77, 53, 0.8 ** np.arange(53), seed=9)
    tol = 1e-4 * np.linalg.norm(A)
    want, got = _both(engine, port, "randQB_pb_new", A, 5, 0, tol, 1, 1)
    assert got[2] == want[2]
    compare_outputs("randQB_pb_new", got, want, rtol=1e-8)


def test_zero_matrix(engine):
    A = np.zeros((64, 40))
    engine.set_omega(SeededOmega(1))
    U, S, V = engine.low_rank_svd_rand_decomp_fixed_rank(A, 8, 4, 1, 2, 1)
    engine.check()
    assert np.all(np.isfinite(U)) and np.all(np.isfinite(V))
    assert np.all(np.diag(S) == 0.0)


@pytest.mark.parametrize("rank", [3, 10])
def test_rank_deficient_input(engine, port, rank):
    """rank(A) < k + p: the Gram of the sketch is singular, so CholeskyQR breaks down and the
    Householder fallback runs; the leading singular values still match the oracle's and the
    trailing ones vanish."""
    m, n, k, p = 120, 90, 12, 4
    g = np.random.default_rng(rank)
    A = g.standard_normal((m, rank)) @ g.standard_normal((rank, n))
    want, got = _both(engine, port, "low_rank_svd_rand_decomp_fixed_rank", A, k, p, 1, 2, 1)
    s_got, s_want = np.diag(got[1]), np.diag(want[1])
    assert np.max(np.abs(s_got[:rank] - s_want[:rank])) <= 1e-10 * s_want[0]
    assert np.max(np.abs(s_got[rank:])) <= 1e-10 * s_want[0]
    U = got[0]
    assert np.max(np.abs(U[:, :rank].T @ U[:, :rank] - np.eye(rank))) < 1e-8


@pytest.mark.parametrize("prec", ["tf32", "fp32"])
def test_rank_deficient_mixed_solve_falls_back(engine, prec):
    """FP32-data solves on Philox test matrices defer each Cholesky's breakdown check to the end
    of the solve; a rank-deficient input breaks CholeskyQR, so the solve is repeated on the same
    test matrices with Householder QR: finite factors, the leading singular values of A, the
    trailing ones near zero, and the same result on a replay of the same draws."""
    m, n, k, p, rank = 3000, 1500, 24, 8, 10
    g = np.random.default_rng(17)
    A = g.standard_normal((m, rank)) @ g.standard_normal((rank, n))
    sv = np.linalg.svd(A, compute_uv=False)
    engine.set_precision(prec)
    engine.set_use_provider(False)
    try:
        runs = []
        for _ in range(2):
            engine.lib.rsvdpack_reset_omega_counter()
            runs.append(engine.low_rank_svd_rand_decomp_fixed_rank(A, k, p, 1, 2, 1))
            engine.check()
    finally:
        engine.set_precision("fp64")
        engine.set_use_provider(True)
    U, S, V = runs[0]
    s = np.diag(S)
    assert np.all(np.isfinite(U)) and np.all(np.isfinite(V)) and np.all(np.isfinite(s))
    # TF32 products carry ~1e-3 relative error (BF16 A in A X); FP32 ~1e-7
    tol = 5e-3 if prec == "tf32" else 1e-5
    assert np.max(np.abs(s[:rank] - sv[:rank]) / sv[:rank]) < tol
    assert np.max(np.abs(s[rank:])) < tol * sv[0]
    assert np.array_equal(runs[0][1], runs[1][1])
