"""The reference's host-side mat / vec helpers (matrix_vector_functions_intel_mkl.c) exported by the
engine: each one run on the same inputs in librsvdpack.so and in the reference's own compiled
helpers (oracle/_ref, where the reference tree is present) must leave identical outputs -- bit for
bit, except vector_dot_product, project_vector, build_orthonormal_basis_from_mat and
get_householder_matrix, whose sums are OpenMP
reductions in the reference (matrix_vector_functions_intel_mkl.c:304,349: the order is set by the
thread count).  Where the reference is absent the same calls
are checked against numpy.  No GPU needed."""
import ctypes as C

import numpy as np
import pytest

from lowrankmatrixdecompositioncodes_gb300 import load_engine

RNG = np.random.default_rng(7)
A0 = RNG.standard_normal((7, 5))
B0 = RNG.standard_normal((7, 5))
V7 = RNG.standard_normal(7)
V5 = RNG.standard_normal(5)
TRUNC = np.array([2.7, -3.2, 0.5, 5.9, -3.9, 5.1, -0.4])     # min / max compare truncated values
PERM7 = np.array([3, 0, 6, 1, 5, 2, 4], dtype=np.float64)
PERM5 = np.array([2, 4, 0, 3, 1], dtype=np.float64)


class Lib:
    """One library, with numpy <-> mat / vec plumbing and the helpers' argtypes."""

    def __init__(self, rl):
        self.rl, self.L = rl, rl.lib
        I, R, PM, PV = rl.Int, rl.Real, rl.PMat, rl.PVec
        sig = {
            "vector_scale": [PV, R], "matrix_scale": [PM, R], "vector_copy": [PV, PV],
            "vector_set_data": [PV, C.POINTER(R)], "matrix_hard_threshold": [PM, R], "vector_sub": [PV, PV],
            "matrix_sub": [PM, PM], "matrix_sub_column_times_row_vector": [PM, PV, PV],
            "vector_get_min_element": [PV, C.POINTER(I), C.POINTER(R)],
            "vector_get_max_element": [PV, C.POINTER(I), C.POINTER(R)],
            "vector_dot_product": [PV, PV], "get_matrix_max_abs_element": [PM],
            "get_matrix_column_norm_squared": [PM, I], "matrix_getmaxcolnorm": [PM],
            "compute_matrix_column_norms": [PM, PV], "invert_diagonal_matrix": [PM, PM],
            "project_vector": [PV, PV, PV], "matrix_get_row": [PM, I, PV], "matrix_set_row": [PM, I, PV],
            "matrix_get_selected_columns": [PM, C.POINTER(I), PM], "matrix_set_selected_columns": [PM, C.POINTER(I), PM],
            "matrix_get_selected_rows": [PM, C.POINTER(I), PM], "matrix_set_selected_rows": [PM, C.POINTER(I), PM],
            "matrix_copy_symmetric": [PM, PM], "matrix_keep_only_upper_triangular": [PM],
            "fill_vector_from_row_list": [PV, PV, PV], "matrix_copy_first_rows": [PM, PM],
            "matrix_copy_first_columns": [PM, PM], "matrix_copy_first_columns_with_param": [PM, PM, I],
            "matrix_copy_first_k_rows_and_columns": [PM, PM],
            "matrix_copy_all_rows_and_last_columns_from_indexk": [PM, PM, I],
            "fill_matrix_from_first_rows": [PM, I, PM], "fill_matrix_from_last_rows": [PM, I, PM],
            "fill_matrix_from_first_columns": [PM, I, PM], "fill_matrix_from_last_columns": [PM, I, PM],
            "fill_matrix_from_last_columns_from_specified_one": [PM, I, PM],
            "fill_matrix_from_lower_right_corner": [PM, I, PM],
            "fill_matrix_from_first_columns_from_list": [PM, PV, I, PM],
            "fill_matrix_from_first_rows_from_list": [PM, PV, I, PM],
            "fill_matrix_from_last_columns_from_list": [PM, PV, I, PM],
            "resize_matrix_by_columns": [C.POINTER(PM), I], "resize_matrix_by_columns_from_end": [C.POINTER(PM), I],
            "resize_matrix_by_rows": [C.POINTER(PM), I], "resize_matrix_by_rows_from_end": [C.POINTER(PM), I],
            "append_matrices_horizontally": [PM, PM, PM], "append_matrices_vertically": [PM, PM, PM],
            "vector_build_rewrapped": [PV, PV], "build_orthonormal_basis_from_mat": [PM, PM],
            "get_householder_matrix": [PV, I, I, PM],
        }
        for name, args in sig.items():
            f = getattr(self.L, name)
            f.argtypes = args
            f.restype = R if name in ("vector_dot_product", "get_matrix_max_abs_element",
                                      "get_matrix_column_norm_squared", "matrix_getmaxcolnorm") else None

    def m(self, A):
        return self.rl.to_mat(A)

    def zeros(self, r, c):
        return self.L.matrix_new(r, c)

    def v(self, x):
        p = self.L.vector_new(len(x))
        for i, t in enumerate(x):
            p.contents.d[i] = t
        return p

    def get(self, p):
        return self.rl.from_mat(p)

    def getv(self, p):
        return self.rl.from_vec(p)

    def ints(self, xs):
        return (self.rl.Int * len(xs))(*[int(t) for t in xs])


def scenario(lib):
    """Runs every helper once; returns the outputs in a dict."""
    L, out = lib.L, {}
    M = lib.m(A0); L.matrix_scale(M, -1.5); out["matrix_scale"] = lib.get(M)
    v = lib.v(V7); L.vector_scale(v, 0.25); out["vector_scale"] = lib.getv(v)
    a, b = lib.v(V7), lib.v(np.zeros(7)); L.vector_copy(b, a); out["vector_copy"] = lib.getv(b); lib.L.vector_delete(a)
    v = lib.v(np.zeros(5)); L.vector_set_data(v, (lib.rl.Real * 5)(*V5)); out["vector_set_data"] = lib.getv(v)
    M = lib.m(A0); L.matrix_hard_threshold(M, 0.7); out["matrix_hard_threshold"] = lib.get(M)
    a, b = lib.v(V7), lib.v(TRUNC); L.vector_sub(a, b); out["vector_sub"] = lib.getv(a); lib.L.vector_delete(b)
    M, N = lib.m(A0), lib.m(B0); L.matrix_sub(M, N); out["matrix_sub"] = lib.get(M); L.matrix_delete(N)
    M, u, w = lib.m(A0), lib.v(V7), lib.v(V5)
    L.matrix_sub_column_times_row_vector(M, u, w); out["matrix_sub_column_times_row_vector"] = lib.get(M)
    t = lib.v(TRUNC)
    for name in ("vector_get_min_element", "vector_get_max_element"):
        idx, val = lib.rl.Int(0), lib.rl.Real(0)
        getattr(L, name)(t, C.byref(idx), C.byref(val))
        out[name] = (idx.value, val.value)
    out["vector_dot_product"] = L.vector_dot_product(u, t)
    M = lib.m(A0)
    out["get_matrix_max_abs_element"] = L.get_matrix_max_abs_element(M)
    out["get_matrix_column_norm_squared"] = L.get_matrix_column_norm_squared(M, 3)
    out["matrix_getmaxcolnorm"] = L.matrix_getmaxcolnorm(M)
    cn = lib.v(np.zeros(5)); L.compute_matrix_column_norms(M, cn); out["compute_matrix_column_norms"] = lib.getv(cn)
    D, Di = lib.m(np.diag(V5 + 3.0)), lib.m(np.full((5, 5), 9.0))
    L.invert_diagonal_matrix(Di, D); out["invert_diagonal_matrix"] = lib.get(Di); L.matrix_delete(D)
    p = lib.v(np.zeros(7)); L.project_vector(t, u, p); out["project_vector"] = lib.getv(p)
    r = lib.v(np.zeros(5)); L.matrix_get_row(M, 4, r); out["matrix_get_row"] = lib.getv(r, )
    N = lib.m(B0); w = lib.v(V5); L.matrix_set_row(N, 2, w); out["matrix_set_row"] = lib.get(N)
    Mc = lib.zeros(7, 3); L.matrix_get_selected_columns(M, lib.ints([4, 0, 2]), Mc); out["get_sel_cols"] = lib.get(Mc)
    N, Mc = lib.m(B0), lib.m(A0[:, :2] * 3)
    L.matrix_set_selected_columns(N, lib.ints([3, 1]), Mc); out["set_sel_cols"] = lib.get(N); L.matrix_delete(Mc)
    Mr = lib.zeros(3, 5); L.matrix_get_selected_rows(M, lib.ints([6, 1, 3]), Mr); out["get_sel_rows"] = lib.get(Mr)
    N, Mr = lib.m(B0), lib.m(A0[:2, :] * 3)
    L.matrix_set_selected_rows(N, lib.ints([5, 0]), Mr); out["set_sel_rows"] = lib.get(N); L.matrix_delete(Mr)
    S = lib.m(np.full((7, 5), -1.0)); L.matrix_copy_symmetric(S, M); out["matrix_copy_symmetric"] = lib.get(S)
    K = lib.m(A0); L.matrix_keep_only_upper_triangular(K); out["matrix_keep_only_upper_triangular"] = lib.get(K)
    o, pi = lib.v(np.zeros(7)), lib.v(PERM7)
    L.fill_vector_from_row_list(t, pi, o); out["fill_vector_from_row_list"] = lib.getv(o)
    for name, shape, extra in (
            ("matrix_copy_first_rows", (3, 5), None), ("matrix_copy_first_columns", (7, 2), None),
            ("matrix_copy_first_columns_with_param", (7, 5), 3), ("matrix_copy_first_k_rows_and_columns", (4, 4), None),
            ("matrix_copy_all_rows_and_last_columns_from_indexk", (7, 3), 2)):
        Z = lib.zeros(*shape)
        if extra is None:
            getattr(L, name)(Z, M)
        else:
            getattr(L, name)(Z, M, extra)
        out[name] = lib.get(Z)
    for name, k, shape in (
            ("fill_matrix_from_first_rows", 3, (3, 5)), ("fill_matrix_from_last_rows", 3, (3, 5)),
            ("fill_matrix_from_first_columns", 2, (7, 2)), ("fill_matrix_from_last_columns", 2, (7, 2)),
            ("fill_matrix_from_last_columns_from_specified_one", 2, (7, 3)),
            ("fill_matrix_from_lower_right_corner", 2, (5, 3))):
        Z = lib.zeros(*shape)
        getattr(L, name)(M, k, Z)
        out[name] = lib.get(Z)
    p5, p7 = lib.v(PERM5), lib.v(PERM7)
    for name, I, k, shape in (
            ("fill_matrix_from_first_columns_from_list", p5, 3, (7, 3)),
            ("fill_matrix_from_first_rows_from_list", p7, 4, (4, 5)),
            ("fill_matrix_from_last_columns_from_list", p5, 2, (7, 3))):
        Z = lib.zeros(*shape)
        getattr(L, name)(M, I, k, Z)
        out[name] = lib.get(Z)
    for name, k in (("resize_matrix_by_columns", 3), ("resize_matrix_by_columns_from_end", 2),
                    ("resize_matrix_by_rows", 4), ("resize_matrix_by_rows_from_end", 3)):
        R = lib.m(A0)
        getattr(L, name)(C.byref(R), k)
        out[name] = lib.get(R)
    Z = lib.zeros(7, 10); N = lib.m(B0); L.append_matrices_horizontally(M, N, Z); out["append_h"] = lib.get(Z)
    Z = lib.zeros(14, 5); L.append_matrices_vertically(M, N, Z); out["append_v"] = lib.get(Z)
    inv = lib.v(np.zeros(7)); L.vector_build_rewrapped(inv, p7); out["vector_build_rewrapped"] = lib.getv(inv)
    Q = lib.zeros(7, 5); L.build_orthonormal_basis_from_mat(M, Q); out["build_orthonormal_basis_from_mat"] = lib.get(Q)
    H = lib.zeros(7, 1); L.get_householder_matrix(u, 2, 7, H); out["get_householder_matrix"] = lib.get(H)
    return out


NOT_EXACT = {"vector_dot_product", "project_vector", "build_orthonormal_basis_from_mat", "get_householder_matrix"}
# the reference's matrix_getmaxcolnorm shares one column buffer and the running maximum between
# OpenMP threads without a reduction (matrix_vector_functions_intel_mkl.c:422-443): its result
# changes from run to run, so it is checked against numpy only
RACY_IN_REFERENCE = {"matrix_getmaxcolnorm"}


def test_helpers_match_the_reference_build(ref):
    got, want = scenario(Lib(load_engine())), scenario(Lib(ref))
    assert got.keys() == want.keys()
    for key in want:
        if key in RACY_IN_REFERENCE:
            continue
        g, w = np.asarray(got[key], dtype=np.float64), np.asarray(want[key], dtype=np.float64)
        if key in NOT_EXACT:
            np.testing.assert_allclose(g, w, rtol=1e-14, atol=0, err_msg=key)
        else:
            assert np.array_equal(g, w), key


def test_helpers_against_numpy():
    out = scenario(Lib(load_engine()))
    assert np.array_equal(out["matrix_scale"], -1.5 * A0)
    assert abs(out["matrix_getmaxcolnorm"] - np.linalg.norm(A0, axis=0).max()) < 1e-14
    assert np.array_equal(out["matrix_sub"], A0 - B0)
    assert np.allclose(out["matrix_sub_column_times_row_vector"], A0 - np.outer(V7, V5))
    assert out["vector_get_min_element"] == (1, -3.0)      # values truncated before comparing
    assert out["vector_get_max_element"] == (3, 5.0)
    assert np.array_equal(out["get_sel_cols"], A0[:, [4, 0, 2]])
    assert np.array_equal(out["get_sel_rows"], A0[[6, 1, 3], :])
    assert np.array_equal(out["matrix_keep_only_upper_triangular"], np.triu(A0))
    assert np.array_equal(out["fill_matrix_from_lower_right_corner"], A0[2:, 2:])
    assert np.array_equal(out["fill_matrix_from_first_rows_from_list"], A0[PERM7[:4].astype(int), :])
    assert np.array_equal(out["fill_matrix_from_last_columns_from_list"], A0[:, PERM5[2:].astype(int)])
    assert np.array_equal(out["resize_matrix_by_rows_from_end"], A0[-3:, :])
    assert np.array_equal(out["append_h"], np.hstack([A0, B0]))
    assert np.array_equal(out["append_v"], np.vstack([A0, B0]))
    inv = out["vector_build_rewrapped"].astype(int)
    assert np.array_equal(PERM7.astype(int)[inv], np.arange(7))
    Q = out["build_orthonormal_basis_from_mat"]
    assert np.allclose(Q.T @ Q, np.eye(5), atol=1e-14)
    Qn, _ = np.linalg.qr(A0)
    assert np.allclose(np.abs(np.sum(Q * Qn, axis=0)), 1.0, atol=1e-12)
    h = out["get_householder_matrix"][:, 0]
    x = np.where(np.arange(7) >= 2, V7, 0.0)
    Hx = x - h * (h @ x)                       # (I - h h^T) x = -+||x|| e_2
    assert np.allclose(Hx[3:], 0, atol=1e-14) and abs(abs(Hx[2]) - np.linalg.norm(x)) < 1e-14
