"""The oracle's decompositions from a given QB (the oneAPI variant's
low_rank_svd_rand_decomp_fromQB / id_rand_decomp_fromQB, restated in oracle/port), pinned
against LAPACK through numpy / scipy: the singular values of B B^T are the squares of B's,
U S V^T reproduces Q B, and the column ID of B uses dgeqp3's pivots with T = R11^-1 R12."""
import numpy as np
import pytest
import scipy.linalg as sl

from conftest import spectrum_matrix


def _qb(m, n, l, seed):
    A = spectrum_matrix(m, n, 0.8 ** np.arange(min(m, n)), seed=seed)
    Q, _ = np.linalg.qr(A @ np.random.default_rng(seed + 1).standard_normal((n, l)))
    return Q, Q.T @ A


@pytest.mark.parametrize("m,n,l", [(300, 200, 40), (150, 400, 60), (90, 90, 30)])
def test_port_svd_from_qb(port, m, n, l):
    Q, B = _qb(m, n, l, seed=m + n)
    U, S, V = port.low_rank_svd_rand_decomp_fromQB(Q, B)
    assert U.shape == (m, l) and S.shape == (l, l) and V.shape == (n, l)
    s = np.diag(S)
    s_ref = np.linalg.svd(B, compute_uv=False)
    assert np.all(np.diff(s) <= 0)
    assert np.max(np.abs(s - s_ref) / s_ref[0]) < 1e-12
    assert np.max(np.abs(U.T @ U - np.eye(l))) < 1e-10
    assert np.linalg.norm(U @ S @ V.T - Q @ B) / np.linalg.norm(Q @ B) < 1e-10


@pytest.mark.parametrize("m,n,l", [(300, 200, 40), (150, 400, 60)])
def test_port_id_from_qb(port, m, n, l):
    Q, B = _qb(m, n, l, seed=3 * m + n)
    I, T = port.id_rand_decomp_fromQB(Q, B)
    _, R, piv = sl.qr(B, mode="economic", pivoting=True)
    assert np.array_equal(I.astype(int), piv)
    k = l
    T_ref = sl.solve_triangular(np.triu(R[:k, :k]), R[:k, k:])
    assert T.shape == (k, n - k)
    assert np.max(np.abs(T - T_ref)) <= 1e-9 * max(1.0, np.max(np.abs(T_ref)))
