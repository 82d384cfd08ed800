"""Streaming load of the reference's binary matrix files into device memory
(rsvdpack_dev_load_binary; the file format of matrix_load_from_binary_file,
matrix_vector_functions_intel_mkl.c:77-133), through the C ABI of all three libraries:

* librsvdpack.so: int32 header, FP64 entries; librsvdpack64.so: int64 header, FP64 entries;
  librsvdpack_f32.so: int64 header, FP32 entries.
* The device matrix (column-major, leading dimension lda >= m) equals the file's matrix exactly in
  FP64, and its round-to-nearest FP32 / BF16 rounding otherwise; a multi-chunk file (above the
  32 MiB chunk) and ragged shapes (not multiples of the 32 x 32 transpose tile).
* The host loader of the C API reads the same file to the same values.
* Errors: a missing file, a leading dimension below m, a truncated file.
"""
import ctypes as C
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

RSVD_DT_F64, RSVD_DT_F32, RSVD_DT_BF16 = 0, 1, 2


def _bind(L):
    L.rsvdpack_dev_load_binary.restype = C.c_int
    L.rsvdpack_dev_load_binary.argtypes = [C.c_char_p, C.c_int, C.c_void_p, C.c_longlong,
                                           C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    L.rsvdpack_binary_file_shape.restype = C.c_int
    L.rsvdpack_binary_file_shape.argtypes = [C.c_char_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]


def _write(path, A, hdr_dtype, val_dtype):
    with open(path, "wb") as f:
        np.array(A.shape, dtype=hdr_dtype).tofile(f)
        np.ascontiguousarray(A, dtype=val_dtype).tofile(f)      # row by row


def _bf16_round(A):
    """Round-to-nearest-even of the file's values to BF16 (8 significant bits) in one step, in FP64
    (rounding FP64 through FP32 first could differ at ties); normal-range values."""
    x = A.astype(np.float64)
    mant, ex = np.frexp(x)                       # x = mant 2^ex, 0.5 <= |mant| < 1
    return np.ldexp(np.rint(np.ldexp(mant, 8)), ex - 8)


def _load(L, path, dtype, m, n, lda):
    tdt = {RSVD_DT_F64: torch.float64, RSVD_DT_F32: torch.float32, RSVD_DT_BF16: torch.bfloat16}[dtype]
    D = torch.full((n, lda), float("nan"), device="cuda", dtype=tdt)   # column-major m x n, ld = lda
    mm, nn = C.c_longlong(0), C.c_longlong(0)
    rc = L.rsvdpack_dev_load_binary(str(path).encode(), dtype, D.data_ptr(), lda, C.byref(mm), C.byref(nn))
    return rc, D, (mm.value, nn.value)


@pytest.fixture(params=["main", "int64", "float"])
def lib(request):
    from lowrankmatrixdecompositioncodes_gb300 import load_engine, load_engine64, load_engine_f32
    if request.param == "main":
        eng, hdr, val = load_engine(), np.int32, np.float64
    elif request.param == "int64":
        eng, hdr, val = load_engine64(), np.int64, np.float64
    else:
        eng, hdr, val = load_engine_f32(), np.int64, np.float32
    _bind(eng.lib)
    return eng, hdr, val


@pytest.mark.parametrize("m,n", [(1000, 777), (37, 5), (20011, 613)])   # the last spans several 32 MiB chunks
def test_load_matches_file(lib, tmp_path, m, n):
    eng, hdr, val = lib
    L = eng.lib
    g = np.random.default_rng(m + n)
    A = (g.standard_normal((m, n)) * np.exp(3 * g.standard_normal((m, 1)))).astype(val)
    path = tmp_path / "a.bin"
    _write(path, A, hdr, val)
    sm, sn = C.c_longlong(0), C.c_longlong(0)
    assert L.rsvdpack_binary_file_shape(str(path).encode(), C.byref(sm), C.byref(sn)) == 0
    assert (sm.value, sn.value) == (m, n)
    lda = m + 3
    t0 = time.perf_counter()
    rc, D, shape = _load(L, path, RSVD_DT_F64, m, n, lda)
    dt = time.perf_counter() - t0
    assert rc == 0, eng.last_error()
    assert shape == (m, n)
    got = D.cpu().numpy()[:, :m].T
    assert np.array_equal(got, A.astype(np.float64))
    assert torch.isnan(D[:, m:]).all(), "wrote beyond the m rows of a column"
    if m * n > 10 ** 7:
        print(f"load {m}x{n} ({A.nbytes / 2**20:.0f} MiB file) into FP64: {dt * 1e3:.1f} ms, "
              f"{A.nbytes / dt / 1e9:.2f} GB/s")
    rc, D, _ = _load(L, path, RSVD_DT_F32, m, n, lda)
    assert rc == 0, eng.last_error()
    assert np.array_equal(D.cpu().numpy()[:, :m].T, A.astype(np.float32))
    rc, D, _ = _load(L, path, RSVD_DT_BF16, m, n, lda)
    assert rc == 0, eng.last_error()
    want = torch.from_numpy(_bf16_round(A).astype(np.float32)).to(torch.bfloat16)   # exact: bf16 values
    assert torch.equal(D.cpu()[:, :m].T, want)


def test_load_agrees_with_the_host_loader(tmp_path):
    from lowrankmatrixdecompositioncodes_gb300 import load_engine
    eng = load_engine()
    L = eng.lib
    _bind(L)
    g = np.random.default_rng(3)
    A = g.standard_normal((300, 200))
    path = tmp_path / "h.bin"
    _write(path, A, np.int32, np.float64)
    L.matrix_load_from_binary_file.restype = C.c_void_p
    L.matrix_load_from_binary_file.argtypes = [C.c_char_p]
    L.matrix_delete.argtypes = [C.c_void_p]
    M = L.matrix_load_from_binary_file(str(path).encode())
    assert M
    try:
        class Mat(C.Structure):
            _fields_ = [("nrows", C.c_int), ("ncols", C.c_int), ("d", C.POINTER(C.c_double))]
        mm = C.cast(M, C.POINTER(Mat)).contents
        host = np.ctypeslib.as_array(mm.d, shape=(200 * 300,)).reshape(200, 300).T.copy()
    finally:
        L.matrix_delete(M)
    rc, D, _ = _load(L, path, RSVD_DT_F64, 300, 200, 300)
    assert rc == 0, eng.last_error()
    assert np.array_equal(D.cpu().numpy().T, host)


def test_load_errors(tmp_path):
    from lowrankmatrixdecompositioncodes_gb300 import load_engine
    eng = load_engine()
    L = eng.lib
    _bind(L)
    D = torch.zeros(4, 64, device="cuda", dtype=torch.float64)
    rc, _, _ = (L.rsvdpack_dev_load_binary(str(tmp_path / "missing.bin").encode(), RSVD_DT_F64, D.data_ptr(), 64,
                                           None, None), None, None)
    assert rc != 0 and "header" in eng.last_error()[1]
    A = np.ones((50, 4))
    path = tmp_path / "t.bin"
    _write(path, A, np.int32, np.float64)
    rc = L.rsvdpack_dev_load_binary(str(path).encode(), RSVD_DT_F64, D.data_ptr(), 40, None, None)
    assert rc != 0 and "leading dimension" in eng.last_error()[1]
    with open(path, "r+b") as f:                     # cut the last row short
        f.truncate(8 + 8 * (50 * 4 - 2))
    rc = L.rsvdpack_dev_load_binary(str(path).encode(), RSVD_DT_F64, D.data_ptr(), 64, None, None)
    assert rc != 0 and "truncated" in eng.last_error()[1]
    # the engine stays usable after the errors
    _write(path, A, np.int32, np.float64)
    rc = L.rsvdpack_dev_load_binary(str(path).encode(), RSVD_DT_F64, D.data_ptr(), 64, None, None)
    assert rc == 0, eng.last_error()
    assert torch.equal(D[:, :50].cpu(), torch.ones(4, 50, dtype=torch.float64))
