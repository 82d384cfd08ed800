"""The C-ABI boundary: librsvdpack.so loads on any machine, exports every function
include/rsvdpack.h declares, and its host-side helpers (mat/vec storage, binary file
format, argument checks, error reporting) behave like the reference's."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from lowrankmatrixdecompositioncodes_gb300 import engine_available, load_engine

HEADER = os.path.join(ROOT, "include", "rsvdpack.h")


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*?[\s\*]+([A-Za-z_][A-Za-z0-9_]*)\s*\(",
                       txt, flags=re.M)
    return sorted({n for n in names if n not in ("if", "return", "typedef", "void")})


def test_header_declares_reference_api():
    names = declared_functions()
    for must in ["low_rank_svd_rand_decomp_fixed_rank", "low_rank_svd_blockrand_decomp_fixed_rank_or_prec",
                 "randQB_pb_new", "id_rand_decomp_fixed_rank", "id_two_sided_rand_decomp_fixed_rank",
                 "cur_rand_decomp_fixed_rank", "pivotedQR_mkl", "matrix_new", "matrix_delete"]:
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = load_engine().lib
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_mat_storage_is_reference_layout():
    eng = load_engine()
    A = np.arange(12, dtype=np.float64).reshape(3, 4)
    M = eng.to_mat(A)
    L = eng.lib
    L.matrix_get_element.restype = C.c_double
    L.matrix_get_element.argtypes = [C.c_void_p, C.c_int, C.c_int]
    assert M.contents.nrows == 3 and M.contents.ncols == 4
    assert L.matrix_get_element(M, 2, 1) == A[2, 1]
    # column-major storage, ld = nrows (matrix_vector_functions_intel_mkl.c:47-55)
    assert M.contents.d[1 * 3 + 2] == A[2, 1]
    back = eng.from_mat(M)
    assert np.array_equal(back, A)


def test_binary_file_round_trip(tmp_path):
    """int32 m, int32 n, then m*n doubles row-major (matrix_vector_functions_intel_mkl.c:77-133)."""
    eng = load_engine()
    L = eng.lib
    L.matrix_load_from_binary_file.restype = C.c_void_p
    L.matrix_load_from_binary_file.argtypes = [C.c_char_p]
    L.matrix_write_to_binary_file.argtypes = [C.c_void_p, C.c_char_p]
    A = np.random.default_rng(0).standard_normal((5, 3))
    f = tmp_path / "a.bin"
    with open(f, "wb") as fh:
        np.array([5, 3], dtype=np.int32).tofile(fh)
        A.astype(np.float64).tofile(fh)          # row-major
    p = L.matrix_load_from_binary_file(str(f).encode())
    from lowrankmatrixdecompositioncodes_gb300.capi import PMat
    pm = C.cast(p, PMat)
    got = eng.from_mat(pm, free=False)
    assert np.array_equal(got, A)
    g = tmp_path / "b.bin"
    L.matrix_write_to_binary_file(p, str(g).encode())
    assert open(f, "rb").read() == open(g, "rb").read()
    eng.lib.matrix_delete(pm)


@pytest.mark.skipif(engine_available(), reason="checks the no-device path")
def test_no_device_fails_loudly_without_outputs():
    eng = load_engine()
    from lowrankmatrixdecompositioncodes_gb300.capi import PMat
    M = eng.to_mat(np.ones((10, 8)))
    U, S, V, fr = PMat(), PMat(), PMat(), C.c_int(0)
    eng.lib.low_rank_svd_rand_decomp_fixed_rank(M, 2, 1, 1, 1, 1, C.byref(fr), C.byref(U), C.byref(S),
                                                C.byref(V))
    code, msg = eng.last_error()
    assert code == 3 and "device" in msg
    assert not U and not S and not V
    eng.lib.matrix_delete(M)


def test_argument_errors_are_reported_not_fatal():
    eng = load_engine()
    from lowrankmatrixdecompositioncodes_gb300.capi import PMat
    M = eng.to_mat(np.ones((10, 8)))
    U, S, V, fr = PMat(), PMat(), PMat(), C.c_int(0)
    # k + p > min(m, n): undefined behaviour in the reference, an error here
    eng.lib.low_rank_svd_rand_decomp_fixed_rank(M, 6, 4, 1, 1, 1, C.byref(fr), C.byref(U), C.byref(S),
                                                C.byref(V))
    code, _ = eng.last_error()
    assert code in (1, 3)   # argument error (or no device, checked first on CPU-only machines)
    assert not U
    eng.lib.matrix_delete(M)
