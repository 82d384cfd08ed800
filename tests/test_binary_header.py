"""rsvdpack_binary_file_shape (host only, no GPU): the header of the reference's binary matrix
files (matrix_vector_functions_intel_mkl.c:77-133) in each library's integer width -- int32 for
librsvdpack.so, int64 for librsvdpack64.so and librsvdpack_f32.so -- and its errors."""
import ctypes as C

import numpy as np
import pytest

from lowrankmatrixdecompositioncodes_gb300 import load_engine, load_engine64, load_engine_f32


@pytest.mark.parametrize("loader,hdr", [(load_engine, np.int32), (load_engine64, np.int64),
                                        (load_engine_f32, np.int64)])
def test_binary_file_shape(tmp_path, loader, hdr):
    eng = loader()
    L = eng.lib
    L.rsvdpack_binary_file_shape.restype = C.c_int
    L.rsvdpack_binary_file_shape.argtypes = [C.c_char_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    p = tmp_path / "a.bin"
    with open(p, "wb") as f:
        np.array([123, 45], dtype=hdr).tofile(f)
    m, n = C.c_longlong(0), C.c_longlong(0)
    assert L.rsvdpack_binary_file_shape(str(p).encode(), C.byref(m), C.byref(n)) == 0
    assert (m.value, n.value) == (123, 45)
    with open(p, "wb") as f:
        np.array([0, 45], dtype=hdr).tofile(f)                 # empty matrix: not a valid file
    assert L.rsvdpack_binary_file_shape(str(p).encode(), C.byref(m), C.byref(n)) != 0
    assert L.rsvdpack_binary_file_shape(str(tmp_path / "none.bin").encode(), C.byref(m), C.byref(n)) != 0
    code, msg = eng.last_error()
    assert code != 0 and "header" in msg
