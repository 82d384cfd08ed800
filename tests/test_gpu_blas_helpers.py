"""GPU checks of the helpers the reference backs with BLAS / LAPACK calls (MVF:532-580,
1477-1531), against numpy: y = M x and M^T x (the FP64 GEMM with one column), the in-place
triangular inverse, the four solve types of upper_triangular_system_solve (type 2 inverts A in
place first) and the LU solve of square_matrix_system_solve (X and B get the solution)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

G = np.random.default_rng(11)
R0 = np.triu(G.standard_normal((40, 40)) * 0.1) + np.diag(G.uniform(1.0, 3.0, 40))
B0 = G.standard_normal((40, 7))


@pytest.fixture
def eng(engine):
    engine.set_precision("fp64")
    L = engine.lib
    L.matrix_vector_mult.argtypes = [engine.PMat, engine.PVec, engine.PVec]
    L.matrix_transpose_vector_mult.argtypes = [engine.PMat, engine.PVec, engine.PVec]
    L.invert_upper_triangular_matrix.argtypes = [engine.PMat]
    L.upper_triangular_system_solve.argtypes = [engine.PMat, engine.PMat, engine.PMat, engine.Int]
    L.square_matrix_system_solve.argtypes = [engine.PMat, engine.PMat, engine.PMat]
    return engine


def _vec(e, x):
    v = e.lib.vector_new(len(x))
    for i, t in enumerate(x):
        v.contents.d[i] = t
    return v


def test_matrix_vector_products(eng):
    M = G.standard_normal((33, 21))
    x, z = G.standard_normal(21), G.standard_normal(33)
    pM, px, py = eng.to_mat(M), _vec(eng, x), _vec(eng, np.zeros(33))
    eng.lib.matrix_vector_mult(pM, px, py)
    eng.check()
    np.testing.assert_allclose(eng.from_vec(py), M @ x, rtol=0, atol=1e-13)
    pz, pw = _vec(eng, z), _vec(eng, np.zeros(21))
    eng.lib.matrix_transpose_vector_mult(pM, pz, pw)
    eng.check()
    np.testing.assert_allclose(eng.from_vec(pw), M.T @ z, rtol=0, atol=1e-13)
    eng.lib.matrix_delete(pM)


def test_triangular_inverse_in_place(eng):
    A = R0 + np.tril(np.full((40, 40), 5.0), -1)          # a strictly lower part that must stay
    pA = eng.to_mat(A)
    eng.lib.invert_upper_triangular_matrix(pA)
    eng.check()
    got = eng.from_mat(pA)
    want = np.linalg.inv(R0)
    np.testing.assert_allclose(np.triu(got), np.triu(want), rtol=0, atol=1e-12)
    assert np.all(got[np.tril_indices(40, -1)] == 5.0)


@pytest.mark.parametrize("solve_type", [0, 1, 2, 3])
def test_upper_triangular_solves(eng, solve_type):
    pA, pB, pX = eng.to_mat(R0), eng.to_mat(B0), eng.lib.matrix_new(40, 7)
    eng.lib.upper_triangular_system_solve(pA, pB, pX, solve_type)
    eng.check()
    np.testing.assert_allclose(eng.from_mat(pX), np.linalg.solve(R0, B0), rtol=0, atol=1e-12)
    Aafter = eng.from_mat(pA)
    if solve_type == 2:                                   # A was inverted in place
        np.testing.assert_allclose(np.triu(Aafter), np.linalg.inv(R0), rtol=0, atol=1e-12)
    else:
        assert np.array_equal(Aafter, R0)
    eng.lib.matrix_delete(pB)


def test_square_system_solve(eng):
    A = G.standard_normal((40, 40)) + 6 * np.eye(40)
    pA, pX, pB = eng.to_mat(A), eng.lib.matrix_new(40, 7), eng.to_mat(B0)
    eng.lib.square_matrix_system_solve(pA, pX, pB)
    eng.check()
    want = np.linalg.solve(A, B0)
    np.testing.assert_allclose(eng.from_mat(pX), want, rtol=0, atol=1e-12)
    np.testing.assert_allclose(eng.from_mat(pB), want, rtol=0, atol=1e-12)
    assert np.array_equal(eng.from_mat(pA), A)


@pytest.mark.parametrize("n", [9, 64, 150])
def test_symmetric_eigensolver(eng, n):
    """compute_evals_and_evecs_of_symm_matrix on an indefinite symmetric matrix whose strictly
    lower part holds other numbers (the upper triangle defines it, as for dsyev 'U')."""
    L = eng.lib
    L.compute_evals_and_evecs_of_symm_matrix.argtypes = [eng.PMat, eng.PVec]
    X = G.standard_normal((n, n))
    Ssym = (X + X.T) / 2
    S = np.triu(Ssym) + np.tril(G.standard_normal((n, n)), -1)
    pS, pe = eng.to_mat(S), _vec(eng, np.zeros(n))
    L.compute_evals_and_evecs_of_symm_matrix(pS, pe)
    eng.check()
    lam, Vec = eng.from_vec(pe), eng.from_mat(pS)
    scale = np.linalg.norm(Ssym)
    np.testing.assert_allclose(lam, np.linalg.eigvalsh(Ssym), rtol=0, atol=1e-12 * scale)
    assert np.all(np.diff(lam) >= -1e-12 * scale)                     # ascending
    assert np.max(np.abs(Vec.T @ Vec - np.eye(n))) < 1e-12
    assert np.max(np.abs(Ssym @ Vec - Vec * lam)) < 1e-11 * scale


def test_symmetric_eigensolver_ill_conditioned(eng):
    """Eigenvalues spread over 12 decades (a graded positive definite matrix, condition 1e12):
    every eigenvalue within ~n eps ||S||_F absolutely of numpy.linalg.eigh (the backward error of
    the FP64 Jacobi on the shifted matrix S + ||S||_F I), and the eigenvectors orthonormal."""
    L = eng.lib
    L.compute_evals_and_evecs_of_symm_matrix.argtypes = [eng.PMat, eng.PVec]
    n = 120
    Qm, _ = np.linalg.qr(G.standard_normal((n, n)))
    lam_true = np.logspace(0, -12, n)
    Ssym = (Qm * lam_true) @ Qm.T
    Ssym = (Ssym + Ssym.T) / 2
    pS, pe = eng.to_mat(Ssym.copy()), _vec(eng, np.zeros(n))
    L.compute_evals_and_evecs_of_symm_matrix(pS, pe)
    eng.check()
    lam, Vec = eng.from_vec(pe), eng.from_mat(pS)
    want = np.linalg.eigvalsh(Ssym)
    fro = np.linalg.norm(Ssym)
    bound = 4 * n * np.finfo(float).eps * fro
    assert np.max(np.abs(lam - want)) < bound
    assert np.max(np.abs(Vec.T @ Vec - np.eye(n))) < 1e-12
    # the large eigenvalues keep their relative accuracy
    np.testing.assert_allclose(lam[-10:], want[-10:], rtol=1e-12)
