"""The allocation-free sketch product (rsvdpack_dev_sketch_t_noalloc), through the C ABI.

It serves callers that cannot allocate GPU memory at the point of the call (an external
memory manager or budget that forbids driver allocations, or code that must avoid the
implicit synchronisation of cudaMalloc / cudaFree): its split-K partial sums live in a
scratch array inside the library instead of in workspace the call would allocate.  Its
result must match the regular entry point (rsvdpack_dev_sketch, TF32 mode) within the
TF32 tolerance, on two calls in a row (the second reuses the scratch the first left
behind), and the device's free memory must not change across calls on a warmed device (the
free-memory test synchronises the whole device first, so it does not depend on the order in
which the suite runs).
"""
import ctypes as C
import warnings

import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TF32_TOL = 3e-3


def _bind(L):
    L.rsvdpack_dev_sketch.restype = C.c_int
    L.rsvdpack_dev_sketch.argtypes = [C.c_void_p, C.c_int, C.c_longlong, C.c_int, C.c_int, C.c_void_p,
                                      C.c_longlong, C.c_int, C.c_void_p, C.c_longlong, C.c_int]
    L.rsvdpack_dev_sketch_t_noalloc.restype = C.c_int
    L.rsvdpack_dev_sketch_t_noalloc.argtypes = [C.c_void_p, C.c_longlong, C.c_int, C.c_int, C.c_void_p,
                                                C.c_longlong, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p]


def _colmajor(rows, cols, ld, gen):
    buf = torch.zeros(cols, ld, device="cuda", dtype=torch.float32)
    buf[:, :rows] = torch.randn(cols, rows, device="cuda", generator=gen)
    return buf


# (3000, 1000, 600): w > 512, so the product runs in three 256-column tiles
@pytest.mark.parametrize("m,n,w", [(4096, 2000, 272), (16384, 8192, 272), (3000, 700, 40), (3000, 1000, 600)])
def test_no_alloc_matches_regular_entry_point_twice(engine, m, n, w):
    L = engine.lib
    _bind(L)
    engine.set_precision("tf32")
    g = torch.Generator(device="cuda")
    g.manual_seed(m + n + w)
    lda = (m + 31) // 32 * 32
    ldy = (n + 31) // 32 * 32
    A = _colmajor(m, n, lda, g)
    X = _colmajor(m, w, lda, g)
    Y_ref = torch.zeros(w, ldy, device="cuda", dtype=torch.float32)
    torch.cuda.synchronize()
    rc = L.rsvdpack_dev_sketch(A.data_ptr(), 1, lda, m, n, X.data_ptr(), lda, w, Y_ref.data_ptr(), ldy, 1)
    assert rc == 0, engine.last_error()
    ref = Y_ref[:, :n]
    scale = float(ref.abs().max())
    # the exact FP64 product as a second anchor
    exact = (A[:, :m].double() @ X[:, :m].double().T).T
    outs = []
    for _ in range(2):
        Y = torch.full((w, ldy), float("nan"), device="cuda", dtype=torch.float32)
        rc = L.rsvdpack_dev_sketch_t_noalloc(A.data_ptr(), lda, m, n, X.data_ptr(), lda, w, Y.data_ptr(), ldy,
                                             None)
        assert rc == 0, engine.last_error()
        got = Y[:, :n]
        err = float((got - ref).abs().max()) / scale
        assert err < TF32_TOL, f"relative difference {err:.3e}"
        assert float((got.double() - exact).abs().max()) / float(exact.abs().max()) < TF32_TOL
        outs.append(got.clone())
    assert torch.equal(outs[0], outs[1]), "the two calls disagree"
    engine.set_precision("fp64")


def test_no_alloc_leaves_free_memory_unchanged(engine):
    """After a warm-up call (which loads the kernel's module, scratch array included), further
    calls change the driver's count of free device memory by nothing."""
    L = engine.lib
    _bind(L)
    m, n, w = 8192, 4096, 272
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    A = _colmajor(m, n, m, g)
    X = _colmajor(m, w, m, g)
    Y = torch.empty(w, n, device="cuda", dtype=torch.float32)
    rc = L.rsvdpack_dev_sketch_t_noalloc(A.data_ptr(), m, m, n, X.data_ptr(), m, w, Y.data_ptr(), n, None)
    assert rc == 0, engine.last_error()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(4):
        rc = L.rsvdpack_dev_sketch_t_noalloc(A.data_ptr(), m, m, n, X.data_ptr(), m, w, Y.data_ptr(), n, None)
        assert rc == 0, engine.last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"


def test_no_alloc_refuses_a_capturing_stream(engine):
    """The call ends by waiting for its stream, so under stream capture it queues nothing and
    returns RSVD_ERR_ARGUMENT; the capture itself ends normally and the call works afterwards."""
    L = engine.lib
    _bind(L)
    m, n, w = 256, 128, 16
    A = torch.zeros(n, m, device="cuda", dtype=torch.float32)
    X = torch.zeros(w, m, device="cuda", dtype=torch.float32)
    Y = torch.zeros(w, n, device="cuda", dtype=torch.float32)
    rc = L.rsvdpack_dev_sketch_t_noalloc(A.data_ptr(), m, m, n, X.data_ptr(), m, w, Y.data_ptr(), n, None)
    assert rc == 0, engine.last_error()          # first call on the device: outside any capture
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(side):
        graph.capture_begin()
        try:
            rc = L.rsvdpack_dev_sketch_t_noalloc(A.data_ptr(), m, m, n, X.data_ptr(), m, w, Y.data_ptr(), n,
                                                 C.c_void_p(side.cuda_stream))
        finally:
            with warnings.catch_warnings():
                warnings.simplefilter("ignore", UserWarning)      # the captured graph is empty, as intended
                graph.capture_end()
    code, msg = engine.last_error()
    assert rc == 1 and code == 1 and "capturing" in msg
    torch.cuda.synchronize()
    rc = L.rsvdpack_dev_sketch_t_noalloc(A.data_ptr(), m, m, n, X.data_ptr(), m, w, Y.data_ptr(), n, None)
    assert rc == 0, engine.last_error()


def test_no_alloc_rejects_products_beyond_its_scratch(engine):
    L = engine.lib
    _bind(L)
    m, n, w = 64, 20000, 512     # round_up(n, 32) * w exceeds the scratch limit
    A = torch.zeros(n, m, device="cuda", dtype=torch.float32)
    X = torch.zeros(w, m, device="cuda", dtype=torch.float32)
    Y = torch.zeros(w, n, device="cuda", dtype=torch.float32)
    rc = L.rsvdpack_dev_sketch_t_noalloc(A.data_ptr(), m, m, n, X.data_ptr(), m, w, Y.data_ptr(), n, None)
    code, msg = engine.last_error()
    assert rc == 1 and code == 1 and "too large" in msg
