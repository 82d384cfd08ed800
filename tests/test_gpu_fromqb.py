"""Decompositions from a given QB on the GPU (low_rank_svd_rand_decomp_fromQB,
id_rand_decomp_fromQB), through the C ABI, against the oracle on the same Q and B (FP64):
singular values to 1e-10 relative, factors up to column sign to 1e-8, pivots exact."""
import numpy as np
import pytest

from conftest import spectrum_matrix

pytestmark = pytest.mark.gpu


def _qb(m, n, l, seed):
    A = spectrum_matrix(m, n, (1.0 + np.arange(min(m, n))) ** -1.5, seed=seed)
    Q, _ = np.linalg.qr(A @ np.random.default_rng(seed + 1).standard_normal((n, l)))
    return Q, Q.T @ A


def _sign_align(X, Y):
    s = np.sign(np.sum(X * Y, axis=0))
    s[s == 0] = 1.0
    return X * s


@pytest.mark.parametrize("m,n,l", [(2000, 1000, 110), (500, 1500, 72), (4096, 2048, 272)])
def test_svd_from_qb_matches_oracle(engine, port, m, n, l):
    engine.set_precision("fp64")
    Q, B = _qb(m, n, l, seed=m + l)
    Ue, Se, Ve = engine.low_rank_svd_rand_decomp_fromQB(Q, B)
    engine.check()
    Up, Sp, Vp = port.low_rank_svd_rand_decomp_fromQB(Q, B)
    se, sp = np.diag(Se), np.diag(Sp)
    assert np.max(np.abs(se - sp) / sp[0]) < 1e-10
    keep = sp > 1e-6 * sp[0]                       # well-separated, well-conditioned columns
    for Xe, Xp in ((Ue, Up), (Ve, Vp)):
        Xe = _sign_align(Xe[:, keep], Xp[:, keep])
        assert np.max(np.abs(Xe - Xp[:, keep])) < 1e-8 * np.max(np.abs(Xp[:, keep]))
    assert np.linalg.norm(Ue @ Se @ Ve.T - Q @ B) / np.linalg.norm(Q @ B) < 1e-10


@pytest.mark.parametrize("m,n,l", [(2000, 1000, 110), (600, 3000, 200)])
def test_id_from_qb_matches_oracle(engine, port, m, n, l):
    engine.set_precision("fp64")
    Q, B = _qb(m, n, l, seed=2 * m + l)
    Ie, Te = engine.id_rand_decomp_fromQB(Q, B)
    engine.check()
    Ip, Tp = port.id_rand_decomp_fromQB(Q, B)
    assert np.array_equal(Ie, Ip)
    assert np.max(np.abs(Te - Tp)) <= 1e-9 * max(1.0, np.max(np.abs(Tp)))
