"""Argument checks of the driver-facing entry points (randQB_pb, randQB_pb2, the QR helpers) in
all three libraries: bad shapes and parameters are reported through rsvdpack_last_error()
(RSVD_ERR_ARGUMENT) with NULL outputs, before any device work -- the reference leaves them
undefined (rank_revealing_algorithms_intel_mkl.c:1425, matrix_vector_functions_intel_mkl.c:1214-1263).
No GPU needed."""
import ctypes as C

import numpy as np
import pytest

from lowrankmatrixdecompositioncodes_gb300 import load_engine, load_engine64, load_engine_f32

LOADERS = {"int": load_engine, "int64": load_engine64, "f32": load_engine_f32}


@pytest.fixture(params=sorted(LOADERS))
def lib(request):
    return LOADERS[request.param]()


def _err(eng):
    code, msg = eng.last_error()
    return code, msg


@pytest.mark.parametrize("kstep,nstep,why", [(0, 2, "kstep"), (4, 0, "nstep"), (8, 2, "exceeds")])
def test_randQB_pb_rejects_bad_blocks(lib, kstep, nstep, why):
    M = lib.to_mat(np.ones((12, 10)))
    Q, B = lib.PMat(), lib.PMat()
    lib.lib.randQB_pb(M, kstep, nstep, 1, 1, C.byref(Q), C.byref(B))
    code, msg = _err(lib)
    assert code == 1 and why in msg
    assert not Q and not B
    lib.lib.matrix_delete(M)


def test_randQB_pb2_checks_like_randQB_pb_new(lib):
    M = lib.to_mat(np.ones((12, 10)))
    Q, B, fr = lib.PMat(), lib.PMat(), lib.Int(0)
    lib.lib.randQB_pb2(M, 0, 1, 0.0, 1, 1, C.byref(fr), C.byref(Q), C.byref(B))
    code, msg = _err(lib)
    assert code == 1 and "randQB_pb2" in msg and "kstep" in msg
    assert not Q and not B
    lib.lib.matrix_delete(M)


def test_qr_helpers_check_shapes(lib):
    L = lib.lib
    L.compact_QR_factorization.argtypes = [lib.PMat, lib.PMat, lib.PMat]
    L.QR_factorization_getQ.argtypes = [lib.PMat, lib.PMat]
    M = lib.to_mat(np.ones((8, 5)))
    Qbad, R = L.matrix_new(8, 4), L.matrix_new(5, 5)
    L.compact_QR_factorization(M, Qbad, R)
    code, msg = _err(lib)
    assert code == 1 and "Q must be m x n" in msg
    Q, Rbad = L.matrix_new(8, 5), L.matrix_new(4, 4)
    L.compact_QR_factorization(M, Q, Rbad)
    code, msg = _err(lib)
    assert code == 1 and "R must be n x n" in msg
    W, QW = lib.to_mat(np.ones((3, 5))), L.matrix_new(3, 5)
    L.QR_factorization_getQ(W, QW)
    code, msg = _err(lib)
    assert code == 1 and "rows >= columns" in msg
    # the caller's buffers are untouched by a rejected call
    assert np.all(lib.from_mat(Q, free=False) == 0) and np.all(lib.from_mat(R, free=False) == 0)
    for x in (M, Qbad, R, Q, Rbad, W, QW):
        L.matrix_delete(x)


def test_identity_and_column_helpers(lib):
    """initialize_identity_matrix, matrix_get_col, matrix_set_col (MVF:504-515, 582-604)."""
    L = lib.lib
    L.initialize_identity_matrix.argtypes = [lib.PMat]
    L.matrix_get_col.argtypes = [lib.PMat, lib.Int, lib.PVec]
    L.matrix_set_col.argtypes = [lib.PMat, lib.Int, lib.PVec]
    D = lib.to_mat(np.full((5, 3), 9.0))
    L.initialize_identity_matrix(D)
    assert np.array_equal(lib.from_mat(D, free=False), np.eye(5, 3, dtype=lib.dtype))
    v = L.vector_new(5)
    for i in range(5):
        v.contents.d[i] = i + 0.5
    L.matrix_set_col(D, 2, v)
    w = L.vector_new(5)
    L.matrix_get_col(D, 2, w)
    assert [w.contents.d[i] for i in range(5)] == [i + 0.5 for i in range(5)]
    got = lib.from_mat(D)
    assert np.array_equal(got[:, 2], np.arange(5) + 0.5) and got[0, 0] == 1 and got[1, 1] == 1
    L.vector_delete(v)
    L.vector_delete(w)


def test_rank_only_pivoted_qr_checks_k(lib):
    M = lib.to_mat(np.ones((6, 4)))
    Q, R, I, fr = lib.PMat(), lib.PMat(), lib.PVec(), lib.Int(0)
    for k in (0, 5):
        lib.lib.pivoted_QR_of_specified_rank(M, k, C.byref(fr), C.byref(Q), C.byref(R), C.byref(I))
        code, msg = _err(lib)
        assert code == 1 and "1 <= k" in msg
        assert not Q and not R and not I
    lib.lib.matrix_delete(M)


def test_older_svd_entry_points_check_arguments(lib):
    L = lib.lib
    for name, n_int in (("randomized_low_rank_svd1", 1), ("randomized_low_rank_svd4", 3)):
        getattr(L, name).argtypes = [lib.PMat] + [lib.Int] * n_int + [C.POINTER(lib.PMat)] * 3
    M = lib.to_mat(np.ones((6, 4)))
    U, S, V = lib.PMat(), lib.PMat(), lib.PMat()
    L.randomized_low_rank_svd1(M, 5, C.byref(U), C.byref(S), C.byref(V))      # k > min(m, n)
    assert _err(lib)[0] == 1 and not U and not S and not V
    L.randomized_low_rank_svd4(M, 2, 0, 1, C.byref(U), C.byref(S), C.byref(V))  # nstep = 0
    code, msg = _err(lib)
    assert code == 1 and "randQB_pb" in msg and not U
    L.matrix_delete(M)


def test_blas_backed_helpers_check_shapes(lib):
    L = lib.lib
    L.invert_upper_triangular_matrix.argtypes = [lib.PMat]
    L.upper_triangular_system_solve.argtypes = [lib.PMat, lib.PMat, lib.PMat, lib.Int]
    L.square_matrix_system_solve.argtypes = [lib.PMat, lib.PMat, lib.PMat]
    W = lib.to_mat(np.ones((4, 3)))
    L.invert_upper_triangular_matrix(W)
    assert _err(lib) == (1, "invert_upper_triangular_matrix: matrix must be square")
    A, B, X = lib.to_mat(np.eye(3)), lib.to_mat(np.ones((3, 2))), lib.to_mat(np.zeros((3, 3)))
    L.upper_triangular_system_solve(A, B, X, 1)
    assert _err(lib)[0] == 1 and "B's shape" in _err(lib)[1]
    L.square_matrix_system_solve(W, X, B)
    assert _err(lib)[0] == 1 and "square A" in _err(lib)[1]
    for x in (W, A, B, X):
        L.matrix_delete(x)
