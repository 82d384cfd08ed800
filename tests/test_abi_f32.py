"""The float-data form of the C ABI (librsvdpack_f32.so): the oneAPI variant's
mat / vec (oneapi_code/matrix_vector_functions_one_api.h:19-32: int64_t dimensions, float data),
float TOL and float returns, its binary file format (int64 m, int64 n, then row-major floats;
matrix_vector_functions_one_api.c:71-130), FP32 as the default precision mode, and the host-side
helpers the oneAPI drivers call.  No GPU needed."""
import ctypes as C

import numpy as np

from lowrankmatrixdecompositioncodes_gb300 import PREC, RsvdOpts, load_engine, load_engine_f32
from lowrankmatrixdecompositioncodes_gb300.capi import MatF32, VecF32
from test_abi import declared_functions


def test_f32_library_exports_every_declared_symbol():
    lib = load_engine_f32().lib
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_f32_layout_elements_and_default_precision():
    assert C.sizeof(MatF32) == 24 and MatF32.d.offset == 16 and C.sizeof(VecF32) == 16
    eng = load_engine_f32()
    L = eng.lib
    A = np.arange(12, dtype=np.float32).reshape(3, 4) / 3
    M = eng.to_mat(A)
    L.matrix_get_element.restype = C.c_float
    L.matrix_get_element.argtypes = [eng.PMat, C.c_int64, C.c_int64]
    assert L.matrix_get_element(M, 2, 1) == A[2, 1]
    assert M.contents.d[1 * 3 + 2] == A[2, 1]
    L.get_matrix_frobenius_norm.restype = C.c_float
    assert abs(L.get_matrix_frobenius_norm(M) - np.linalg.norm(A.astype(np.float64))) < 1e-6
    got = eng.from_mat(M)
    assert got.dtype == np.float32 and np.array_equal(got, A)
    o = RsvdOpts()
    L.rsvdpack_get_opts(C.byref(o))
    assert o.precision == PREC["fp32"]
    o64 = RsvdOpts()
    load_engine().lib.rsvdpack_get_opts(C.byref(o64))
    assert o64.precision == PREC["fp64"]


def test_f32_binary_file_format(tmp_path):
    eng = load_engine_f32()
    L = eng.lib
    L.matrix_load_from_binary_file.restype = eng.PMat
    L.matrix_load_from_binary_file.argtypes = [C.c_char_p]
    L.matrix_write_to_binary_file.argtypes = [eng.PMat, C.c_char_p]
    A = np.random.default_rng(4).standard_normal((5, 7)).astype(np.float32)
    f = tmp_path / "f.bin"
    with open(f, "wb") as fh:
        np.array([5, 7], dtype=np.int64).tofile(fh)
        A.tofile(fh)
    pm = L.matrix_load_from_binary_file(str(f).encode())
    assert pm and np.array_equal(eng.from_mat(pm, free=False), A)
    g = tmp_path / "g.bin"
    L.matrix_write_to_binary_file(pm, str(g).encode())
    assert open(f, "rb").read() == open(g, "rb").read()
    L.matrix_delete(pm)


def test_diagonal_and_vector_norm_helpers():
    """initialize_diagonal_matrix and vector_get2norm (MVF:490-499, 299-311) in both element types."""
    for eng, ctype in ((load_engine(), C.c_double), (load_engine_f32(), C.c_float)):
        L = eng.lib
        L.initialize_diagonal_matrix.argtypes = [eng.PMat, eng.PVec]
        L.vector_get2norm.argtypes = [eng.PVec]
        L.vector_get2norm.restype = ctype
        v = L.vector_new(4)
        vals = [3.0, -4.0, 12.0, 0.5]
        for i, x in enumerate(vals):
            v.contents.d[i] = x
        D = L.matrix_new(4, 4)
        D.contents.d[1] = 9.0                    # off-diagonal entries are left as they are
        L.initialize_diagonal_matrix(D, v)
        got = eng.from_mat(D)
        want = np.diag(vals)
        want[1, 0] = 9.0
        assert np.array_equal(got, want.astype(eng.dtype))
        assert abs(L.vector_get2norm(v) - np.linalg.norm(vals)) < 1e-6
        L.vector_delete(v)
