"""GPU checks of the QB / QR entry points the oneAPI and MKL drivers call, and of the float-data
library (librsvdpack_f32.so, the oneAPI variant's ABI) against the double-data one.

* randQB_pb (rank_revealing_algorithms_intel_mkl.c:1425-1570: every block after the first
  re-orthogonalised) against the oracle on the same test matrices, FP64 (factors to 1e-8);
  randQB_pb2 (oneapi_code/rank_revealing_algorithms_one_api.c:605-815) gives randQB_pb_new's
  outputs exactly.
* QR_factorization_getQ / compact_QR_factorization (MVF:1214-1263): LAPACK's reflector signs,
  so Q and R match numpy's (LAPACK dgeqrf / dorgqr) to rounding, column signs included.
* librsvdpack_f32.so computes in FP32 by default; on a float-representable matrix its outputs
  are the double library's FP32-mode outputs rounded to float (the same device data, the same
  kernels; checked to 4 float ulps of each output's largest entry), and its FP64 mode gives the
  double library's FP64 outputs rounded to float, with identical pivot sets and ranks.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import spectrum_matrix
from lowrankmatrixdecompositioncodes_gb300 import PREC, RsvdOpts, load_engine_f32
from lowrankmatrixdecompositioncodes_gb300.capi import SeededOmega
from parity import compare_outputs

pytestmark = pytest.mark.gpu


def _seeded(lib, seed):
    lib.set_omega(SeededOmega(seed))
    lib.lib.rsvdpack_reset_omega_counter()


@pytest.mark.parametrize("shape,args", [((300, 200), (16, 4, 1, 1)), ((200, 300), (10, 6, 2, 2))])
def test_randQB_pb_matches_oracle(engine, port, shape, args):
    engine.set_precision("fp64")
    engine.set_use_provider(True)
    A = spectrum_matrix(*shape, 0.93 ** np.arange(min(shape)), seed=sum(shape))
    outs = []
    for lib in (port, engine):
        _seeded(lib, 4)
        outs.append(lib.randQB_pb(A, *args))
    engine.check()
    compare_outputs("randQB_pb", outs[1], outs[0], rtol=1e-8)
    Q, B = outs[1]
    kstep, nstep = args[0], args[1]
    assert Q.shape == (shape[0], kstep * nstep) and B.shape == (kstep * nstep, shape[1])
    assert np.max(np.abs(Q.T @ Q - np.eye(Q.shape[1]))) < 1e-12


def test_randQB_pb2_is_randQB_pb_new(engine):
    engine.set_precision("fp64")
    engine.set_use_provider(True)
    A = spectrum_matrix(256, 192, 0.9 ** np.arange(192), seed=12)
    tol = 1e-5 * np.linalg.norm(A)
    _seeded(engine, 8)
    Q1, B1, f1 = engine.randQB_pb_new(A, 16, 0, tol, 1, 1)
    _seeded(engine, 8)
    Q2, B2, f2 = engine.randQB_pb2(A, 16, 0, tol, 1, 1)
    engine.check()
    assert f1 == f2 > 0
    assert np.array_equal(Q1, Q2) and np.array_equal(B1, B2)


@pytest.mark.parametrize("shape", [(200, 64), (333, 333), (1000, 40)])
def test_householder_qr_entry_points_match_lapack(engine, shape):
    m, n = shape
    A = np.random.default_rng(m + n).standard_normal(shape)
    Qn, Rn = np.linalg.qr(A)
    L = engine.lib
    L.compact_QR_factorization.argtypes = [engine.PMat, engine.PMat, engine.PMat]
    L.QR_factorization_getQ.argtypes = [engine.PMat, engine.PMat]
    M = engine.to_mat(A)
    Q, R, Q2 = L.matrix_new(m, n), L.matrix_new(n, n), L.matrix_new(m, n)
    for i in range(n):                       # the strict lower part of R is left as it is
        for j in range(i):
            R.contents.d[j * n + i] = 7.0
    L.compact_QR_factorization(M, Q, R)
    engine.check()
    L.QR_factorization_getQ(M, Q2)
    engine.check()
    Qe, Re, Qe2 = engine.from_mat(Q), engine.from_mat(R), engine.from_mat(Q2)
    L.matrix_delete(M)
    assert np.max(np.abs(Qe - Qn)) < 1e-11 and np.array_equal(Qe, Qe2)
    assert np.max(np.abs(np.triu(Re) - Rn)) < 1e-11 * np.abs(Rn).max()
    assert np.all(Re[np.tril_indices(n, -1)] == 7.0)


def test_qr_entry_points_reject_wide_input(engine):
    L = engine.lib
    L.QR_factorization_getQ.argtypes = [engine.PMat, engine.PMat]
    M, Q = engine.to_mat(np.ones((4, 6))), L.matrix_new(4, 6)
    L.QR_factorization_getQ(M, Q)
    assert engine.last_error()[0] == 1
    L.matrix_delete(M)
    L.matrix_delete(Q)


def _f32_lib():
    e = load_engine_f32()
    e.set_use_provider(True)
    return e


def test_f32_library_defaults_to_fp32_and_matches_the_double_library(engine):
    ef = _f32_lib()
    o = RsvdOpts()
    ef.lib.rsvdpack_get_opts(C.byref(o))
    assert o.precision == PREC["fp32"]
    A = spectrum_matrix(640, 400, 0.92 ** np.arange(400), seed=31).astype(np.float32)
    engine.set_precision("fp32")
    engine.set_use_provider(True)
    outs = []
    for lib in (engine, ef):
        _seeded(lib, 21)
        outs.append(lib.low_rank_svd_rand_decomp_fixed_rank(A, 30, 10, 1, 2, 1))
        lib.check()
    (U1, S1, V1), (U2, S2, V2) = outs
    assert U2.dtype == np.float32 and S2.dtype == np.float32
    _same_to_float(U2, U1)
    _same_to_float(V2, V1)
    _same_to_float(S2, S1)
    engine.set_precision("fp64")


def _same_to_float(x32, x64):
    """x32 is x64 rounded to float (a few ulps allowed for a reduction order that differs)."""
    ref = x64.astype(np.float32)
    assert x32.shape == ref.shape
    scale = float(np.abs(ref).max()) if ref.size else 0.0
    assert float(np.abs(x32.astype(np.float64) - ref.astype(np.float64)).max()) <= 4 * np.finfo(np.float32).eps * scale


def test_f32_library_fp64_mode_and_id_qb(engine):
    ef = _f32_lib()
    ef.set_precision("fp64")
    engine.set_precision("fp64")
    engine.set_use_provider(True)
    A = spectrum_matrix(500, 360, 0.9 ** np.arange(360), seed=41).astype(np.float32)
    try:
        res = []
        for lib in (engine, ef):
            _seeded(lib, 2)
            I, T = lib.id_rand_decomp_fixed_rank(A, 25, 10, 2, 1)
            _seeded(lib, 3)
            Q, B, f = lib.randQB_pb2(A, 16, 0, 1e-4 * float(np.linalg.norm(A)), 1, 1)
            lib.check()
            res.append((I, T, Q, B, f))
        (I1, T1, Q1, B1, f1), (I2, T2, Q2, B2, f2) = res
        assert np.array_equal(I2, I1.astype(np.float32))
        _same_to_float(T2, T1)
        # TOL is a float in the oneAPI ABI: the same rank when the float TOL does not change
        # the step at which the residual drops below it
        assert f1 == f2
        _same_to_float(Q2, Q1)
        _same_to_float(B2, B1)
    finally:
        ef.set_precision("fp32")
