"""Profiling cases for ncu: each runs one kernel family of the engine on a fixed case,
warm-up calls first, then exactly one call bracketed by cudaProfilerStart / cudaProfilerStop
(capture with ``ncu --profile-from-start off``).  Sizes keep the device footprint to a few
GB and the operands larger than L2 (129 MB), so DRAM counters stay meaningful.

  update   C (8192 x 16384) -= A^T X, K = 256   (blocked-QB deflation, rsvdpack_dev_update_3xtf32)
  gemm3x   D (16384 x 256) = A^T X, K = 16384   (B = Q^T A of the block loop, rsvdpack_dev_gemm_3xtf32)
  solve    one fixed-rank TF32 solve, 16384 x 8192, k = 256, p = 16, q = 2 (the Jacobi SVD,
           Cholesky and product kernels of the headline workload)
  pivot    pivotedQR_mkl of a 520 x 10000 FP64 matrix through the C API (the row sketch of the
           two-sided ID / CUR workload: the column-norm, pivot-select and reflector-apply
           sweeps)
  norm     the Frobenius-norm sweep of the plain FP32 blocked QB (rsvdpack_dev_qb, TOL mode,
           one block) on a 32768 x 16384 FP32 matrix (2 GiB)

    python -m lowrankmatrixdecompositioncodes_gb300.prof_cases update
"""
from __future__ import annotations

import ctypes as C
import sys


def _engine():
    from . import load_engine
    eng = load_engine()
    sms, _, cc = eng.device_info()
    if sms <= 0 or cc != (10, 3):
        raise RuntimeError(f"no GB300 visible: {eng.last_error()}")
    return eng


def _run(torch, fn, warm=2):
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()
    fn()
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStop()


def case_update(torch, eng):
    L = eng.lib
    L.rsvdpack_dev_update_3xtf32.argtypes = [C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong, C.c_int, C.c_int,
                                             C.c_int, C.c_void_p, C.c_longlong, C.POINTER(C.c_double)]
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    M, N, K = 8192, 16384, 256
    A = torch.randn(M, K, device="cuda", generator=g)       # K x M column-major
    X = torch.randn(N, K, device="cuda", generator=g)       # K x N column-major
    Cm = torch.randn(N, M, device="cuda", generator=g)      # M x N column-major
    f2 = C.c_double(0)

    def call():
        if L.rsvdpack_dev_update_3xtf32(A.data_ptr(), K, X.data_ptr(), K, M, N, K, Cm.data_ptr(), M, C.byref(f2)):
            raise RuntimeError(eng.last_error())
    _run(torch, call)


def case_gemm3x(torch, eng):
    L = eng.lib
    L.rsvdpack_dev_gemm_3xtf32.argtypes = [C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong, C.c_int, C.c_int,
                                           C.c_int, C.c_void_p, C.c_longlong]
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    M, N, K = 16384, 256, 16384
    A = torch.randn(M, K, device="cuda", generator=g)
    X = torch.randn(N, K, device="cuda", generator=g)
    D = torch.empty(N, M, device="cuda")

    def call():
        if L.rsvdpack_dev_gemm_3xtf32(A.data_ptr(), K, X.data_ptr(), K, M, N, K, D.data_ptr(), M):
            raise RuntimeError(eng.last_error())
    _run(torch, call)


def case_solve(torch, eng):
    L = eng.lib
    L.rsvdpack_dev_svd_fixed_rank.restype = C.c_int
    L.rsvdpack_dev_svd_fixed_rank.argtypes = [C.c_void_p, C.c_int, C.c_longlong, C.c_int, C.c_int, C.c_int, C.c_int,
                                              C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p,
                                              C.c_void_p, C.c_longlong]
    eng.set_precision("tf32")
    eng.set_use_provider(False)
    m, n, k, p = 16384, 8192, 256, 16
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    U0, _ = torch.linalg.qr(torch.randn(m, n, device="cuda", generator=g))
    V0, _ = torch.linalg.qr(torch.randn(n, n, device="cuda", generator=g))
    s = torch.arange(1, n + 1, device="cuda", dtype=torch.float32) ** -1.5
    At = ((U0 * s) @ V0.T + 1e-4 * torch.randn(m, n, device="cuda", generator=g)).T.contiguous()
    torch.backends.cuda.matmul.allow_tf32 = prev
    del U0, V0
    U = torch.empty(k, m, device="cuda")
    V = torch.empty(k, n, device="cuda")
    S = torch.empty(k, device="cuda", dtype=torch.float64)

    def call():
        if L.rsvdpack_dev_svd_fixed_rank(At.data_ptr(), 1, m, m, n, k, p, 1, 2, 1, U.data_ptr(), m, S.data_ptr(),
                                         V.data_ptr(), n):
            raise RuntimeError(eng.last_error())
    _run(torch, call)


def case_pivot(torch, eng):
    import numpy as np
    eng.set_precision("fp64")
    A = np.random.default_rng(2).standard_normal((520, 10000))

    def call():
        eng.pivotedQR_mkl(A)
        eng.check()
    _run(torch, call, warm=1)


def case_norm(torch, eng):
    L = eng.lib
    L.rsvdpack_dev_qb.restype = C.c_int
    L.rsvdpack_dev_qb.argtypes = [C.c_void_p, C.c_int, C.c_longlong, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                  C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong, C.c_int,
                                  C.POINTER(C.c_int)]
    eng.set_precision("fp32")
    eng.set_learned(False)
    m, n, cap = 32768, 16384, 64
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    At = torch.randn(n, m, device="cuda", generator=g)
    Q = torch.empty(cap, m, device="cuda")
    B = torch.empty(n, cap, device="cuda")
    tol = 0.999 * float(torch.linalg.norm(At.double()))           # stops after the first block
    fr = C.c_int(0)

    def call():
        if L.rsvdpack_dev_qb(At.data_ptr(), 1, m, m, n, 64, 0, tol, 1, 1, Q.data_ptr(), m, B.data_ptr(), cap, cap,
                             C.byref(fr)):
            raise RuntimeError(eng.last_error())
    _run(torch, call)


CASES = {"update": case_update, "gemm3x": case_gemm3x, "solve": case_solve, "pivot": case_pivot, "norm": case_norm}


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) != 1 or argv[0] not in CASES:
        raise SystemExit(f"usage: python -m lowrankmatrixdecompositioncodes_gb300.prof_cases {{{','.join(CASES)}}}")
    import torch
    eng = _engine()
    CASES[argv[0]](torch, eng)
    print("ok", argv[0])


if __name__ == "__main__":
    main()
