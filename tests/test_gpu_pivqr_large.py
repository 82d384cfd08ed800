"""The reference's own deterministic pivoted QR (pivoted_QR_of_specified_rank_or_prec,
multi_core_mkl_code/rank_revealing_algorithms_intel_mkl.c:1159-1334) and the ID built on it
(id_decomp_fixed_rank_or_prec, :1807-1854) at 2000 x 1000, rank 200, through the C ABI against
the oracle: the pivot order identical, R and T to 1e-8 of their largest entry, Q's leading columns
equal up to sign; both timed (the reference forms an explicit m x m Q by rank-1 updates, the engine
forms Q from the stored reflectors)."""
import time

import numpy as np
import pytest

from conftest import spectrum_matrix

pytestmark = pytest.mark.gpu

M, N, K = 2000, 1000, 200


@pytest.fixture(scope="module")
def matrix():
    g = np.random.default_rng(12)
    A = spectrum_matrix(M, N, 0.99 ** np.arange(N), seed=12)
    return A * np.exp(0.5 * g.standard_normal(N))        # uneven column norms


def test_pivoted_qr_rank_mode_matches_oracle_at_scale(engine, port, matrix):
    engine.set_precision("fp64")
    t0 = time.perf_counter()
    Qo, Ro, Io, fo = port.pivoted_QR_of_specified_rank_or_prec(matrix, K, 0.0)
    t1 = time.perf_counter()
    Qe, Re, Ie, fe = engine.pivoted_QR_of_specified_rank_or_prec(matrix, K, 0.0)
    t2 = time.perf_counter()
    engine.check()
    print(f"pivoted QR 2000x1000 rank 200: oracle {t1 - t0:.2f} s, engine {t2 - t1:.2f} s")
    assert fe == fo == K
    assert np.array_equal(Ie, Io), "pivot order differs"
    assert Re.shape == Ro.shape
    r = min(K, Re.shape[0])
    scale = np.max(np.abs(Ro))
    # rows of R and columns of Q may differ in sign together
    sgn = np.sign(np.diag(Re)[:r]) * np.sign(np.diag(Ro)[:r])
    assert np.max(np.abs(Re[:r] * sgn[:, None] - Ro[:r])) < 1e-8 * scale
    assert np.max(np.abs(Qe[:, :r] * sgn - Qo[:, :r])) < 1e-8


def test_deterministic_id_matches_oracle_at_scale(engine, port, matrix):
    engine.set_precision("fp64")
    t0 = time.perf_counter()
    Io, To, fo = port.id_decomp_fixed_rank_or_prec(matrix, K, 0.0)
    t1 = time.perf_counter()
    Ie, Te, fe = engine.id_decomp_fixed_rank_or_prec(matrix, K, 0.0)
    t2 = time.perf_counter()
    engine.check()
    print(f"deterministic ID 2000x1000 rank 200: oracle {t1 - t0:.2f} s, engine {t2 - t1:.2f} s")
    assert fe == fo == K
    assert np.array_equal(Ie, Io)
    assert np.max(np.abs(Te - To)) < 1e-8 * max(1.0, np.max(np.abs(To)))
