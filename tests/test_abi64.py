"""The int64_t-index form of the C ABI (librsvdpack64.so): the reference's 64-bit variant
(multi_core_mkl_code_64bit/matrix_vector_functions_intel_mkl.h:20-28, int64_t dimensions and
int64_t rank / step / frank arguments in rank_revealing_algorithms_intel_mkl.h) over the same
engine.  These checks need no GPU: the library loads, exports every declared function, lays
mat / vec out with 8-byte dimensions, reads and writes the variant's binary file format
(int64 m, int64 n, then row-major doubles; matrix_vector_functions_intel_mkl.c:86-87,123-124)
and rejects arguments the int-dimension engine cannot take before touching any data."""
import ctypes as C

import numpy as np

from lowrankmatrixdecompositioncodes_gb300 import load_engine, load_engine64
from lowrankmatrixdecompositioncodes_gb300.capi import Mat64, Vec64
from test_abi import declared_functions


def test_library64_exports_every_declared_symbol():
    lib = load_engine64().lib
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_mat64_layout_and_element_access():
    assert C.sizeof(Mat64) == 24 and Mat64.d.offset == 16
    assert C.sizeof(Vec64) == 16 and Vec64.d.offset == 8
    eng = load_engine64()
    L = eng.lib
    A = np.arange(12, dtype=np.float64).reshape(3, 4)
    M = eng.to_mat(A)
    assert M.contents.nrows == 3 and M.contents.ncols == 4
    L.matrix_get_element.restype = C.c_double
    L.matrix_get_element.argtypes = [eng.PMat, C.c_int64, C.c_int64]
    L.matrix_set_element.argtypes = [eng.PMat, C.c_int64, C.c_int64, C.c_double]
    assert L.matrix_get_element(M, 2, 1) == A[2, 1]
    L.matrix_set_element(M, 1, 3, -7.5)
    assert M.contents.d[3 * 3 + 1] == -7.5       # column-major, ld = nrows
    v = L.vector_new(5)
    assert v.contents.nrows == 5
    L.vector_delete(v)
    assert np.array_equal(eng.from_mat(M)[0], A[0])


def test_binary_file_int64_header(tmp_path):
    eng = load_engine64()
    L = eng.lib
    L.matrix_load_from_binary_file.restype = eng.PMat
    L.matrix_load_from_binary_file.argtypes = [C.c_char_p]
    L.matrix_write_to_binary_file.argtypes = [eng.PMat, C.c_char_p]
    A = np.random.default_rng(1).standard_normal((4, 6))
    f = tmp_path / "a64.bin"
    with open(f, "wb") as fh:
        np.array([4, 6], dtype=np.int64).tofile(fh)
        A.tofile(fh)                                 # row-major
    pm = L.matrix_load_from_binary_file(str(f).encode())
    assert pm and pm.contents.nrows == 4 and pm.contents.ncols == 6
    got = eng.from_mat(pm, free=False)
    assert np.array_equal(got, A)
    g = tmp_path / "b64.bin"
    L.matrix_write_to_binary_file(pm, str(g).encode())
    assert open(f, "rb").read() == open(g, "rb").read()
    L.matrix_delete(pm)


def test_host_helpers_agree_with_the_int_library():
    e32, e64 = load_engine(), load_engine64()
    A = np.random.default_rng(2).standard_normal((37, 11))
    B = A + 1e-3 * np.random.default_rng(3).standard_normal(A.shape)
    a32, b32, a64, b64 = e32.to_mat(A), e32.to_mat(B), e64.to_mat(A), e64.to_mat(B)
    assert e32.lib.get_matrix_frobenius_norm(a32) == e64.lib.get_matrix_frobenius_norm(a64)
    assert (e32.lib.get_percent_error_between_two_mats(a32, b32)
            == e64.lib.get_percent_error_between_two_mats(a64, b64))
    for e, m in ((e32, a32), (e32, b32), (e64, a64), (e64, b64)):
        e.lib.matrix_delete(m)


def test_out_of_int_range_arguments_are_rejected():
    eng = load_engine64()
    L = eng.lib
    M = eng.to_mat(np.ones((10, 8)))
    U, S, V, fr = eng.PMat(), eng.PMat(), eng.PMat(), C.c_int64(0)
    # a rank above 2^31 - 1 cannot reach the int-dimension engine
    L.low_rank_svd_rand_decomp_fixed_rank(M, 1 << 40, 1, 1, 1, 1, C.byref(fr), C.byref(U), C.byref(S), C.byref(V))
    code, msg = eng.last_error()
    assert code == 1 and "int range" in msg
    assert not U and not S and not V
    L.matrix_delete(M)
    # a dimension above 2^31 - 1 is refused before the data pointer is read
    one = (C.c_double * 1)(0.0)
    big = Mat64(1 << 31, 2, C.cast(one, C.POINTER(C.c_double)))
    Q, B, fr = eng.PMat(), eng.PMat(), C.c_int64(0)
    L.randQB_pb_new(C.byref(big), 1, 1, 0.0, 1, 1, C.byref(fr), C.byref(Q), C.byref(B))
    code, msg = eng.last_error()
    assert code == 1 and "2^31" in msg
    assert not Q and not B
