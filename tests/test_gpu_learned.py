"""The learned fixed-precision QB (randQB_pb_new in TOL mode, rsvdpack_opts.learned): the
proposal's block loop must meet the tolerance exactly as the reference's criterion states
(||A - Q B||_F <= TOL, checked here in FP64), keep Q orthonormal, and keep going when the
proposal underestimates.  A constant network (zero weights, output bias log2(W / 32)) pins
the proposed width W, so these tests do not depend on training; the trained network's gain
over the plain loop is measured in test_trained_proposal_beats_the_plain_loop."""
import ctypes as C
import os
import time

import numpy as np
import pytest

from conftest import spectrum_matrix

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "..", "lowrankmatrixdecompositioncodes_gb300", "learned", "proposal_mlp.bin")


def _constant_model(engine, width):
    L = engine.lib
    dims = (C.c_int * 4)()
    npar = C.c_int(0)
    assert L.rsvdpack_mlp_info(dims, C.byref(npar)) == 0
    P = np.zeros(npar.value, np.float32)
    P[-dims[3]:] = np.log2(width / 32.0)            # output bias
    norm = np.concatenate([np.zeros(dims[0]), np.ones(dims[0])]).astype(np.float32)
    margin = np.zeros(dims[3], np.float32)
    f = C.POINTER(C.c_float)
    L.rsvdpack_set_proposal_model.argtypes = [f, C.c_int, f, C.c_int, f, C.c_int]
    rc = L.rsvdpack_set_proposal_model(P.ctypes.data_as(f), P.size, norm.ctypes.data_as(f), norm.size,
                                       margin.ctypes.data_as(f), margin.size)
    assert rc == 0, engine.last_error()


def _qb(engine, A, tol_abs, learned, prec, kstep=64, q=1):
    engine.set_precision(prec)
    engine.set_learned(learned)
    try:
        Q, B, f = engine.randQB_pb_new(A, kstep, 0, tol_abs, q, 1)
    except ValueError:                                   # NULL outputs: the engine reported an error
        raise RuntimeError(engine.last_error())
    engine.check()
    path = engine.last_timing().learned_path
    engine.set_learned(False)
    engine.set_precision("fp64")
    return Q, B, f, path


@pytest.mark.parametrize("width", [640, 96])
def test_learned_qb_meets_the_tolerance(engine, width):
    m, n = 3000, 1500
    A = spectrum_matrix(m, n, np.exp(-np.arange(n) / 40.0), seed=21)
    # 1e-5: FP32 arithmetic certifies residuals down to ~sqrt(m/8) * 2^-24 of ||A|| (the
    # accumulation of B = Q^T A over m rows); 1e-6 is below that floor for m = 3000
    tol = 1e-5 * np.linalg.norm(A)
    _constant_model(engine, width)
    Q, B, f, path = _qb(engine, A, tol, True, "tf32")
    assert path == 1, "the learned block loop did not run to the tolerance"
    res = np.linalg.norm(A - Q @ B)
    assert res <= tol * (1 + 1e-3), (res, tol, f)
    assert np.max(np.abs(Q.T @ Q - np.eye(f))) < 1e-4
    # the optimal rank for this tolerance, and what the plain loop needs
    s = np.exp(-np.arange(n) / 40.0)
    tail = np.sqrt(np.maximum(np.sum(s * s) - np.cumsum(s * s), 0) / np.sum(s * s))
    k_opt = int(np.searchsorted(-tail, -1e-5)) + 1
    assert k_opt <= f <= k_opt + 4 * max(width // 2, 32) + 64, (k_opt, f)


def test_learned_flag_is_ignored_in_fp64(engine):
    A = spectrum_matrix(800, 500, np.exp(-np.arange(500) / 20.0), seed=3)
    _constant_model(engine, 256)
    _, _, _, path = _qb(engine, A, 1e-5 * np.linalg.norm(A), True, "fp64")
    assert path == 0


@pytest.mark.skipif(not os.path.exists(WEIGHTS), reason="no trained proposal weights")
def test_trained_proposal_beats_the_plain_loop(engine):
    """Same matrices and tolerances: the plain FP32 adaptive loop (the reference algorithm,
    kstep = 64, q = 1) against the learned blocked loop in TF32 mode.  Both must meet the
    tolerance; the learned one must take fewer passes over A and less time overall."""
    engine.load_proposal_model(WEIGHTS)
    g = np.random.default_rng(8)
    cases = [(4096, 2048, np.exp(-np.arange(2048) / 60.0), 1e-5),
             (4096, 2048, (1.0 + np.arange(2048)) ** -3.0, 1e-5),
             (3000, 3000, np.exp(-np.arange(3000) / 25.0), 1e-5),
             (5000, 1800, np.exp(-np.arange(1800) / 120.0), 1e-4)]
    t_plain = t_learned = 0.0
    for i, (m, n, s, tr) in enumerate(cases):
        A = spectrum_matrix(m, n, s, seed=100 + i)
        tol = tr * np.linalg.norm(A)
        for learned, prec in ((False, "fp32"), (True, "tf32")):
            _qb(engine, A, tol, learned, prec)                      # warm-up
            t0 = time.perf_counter()
            Q, B, f, path = _qb(engine, A, tol, learned, prec)
            dt = time.perf_counter() - t0
            res = np.linalg.norm(A - Q @ B)
            assert res <= tol * (1 + 1e-3), (i, learned, res, tol)
            if learned:
                t_learned += dt
                assert path == 1
            else:
                t_plain += dt
            print(f"case {i}: {'learned' if learned else 'plain  '} rank {f:5d} {dt * 1e3:8.1f} ms")
    print(f"plain {t_plain * 1e3:.1f} ms, learned {t_learned * 1e3:.1f} ms, speed-up {t_plain / t_learned:.2f}x")
    assert t_learned < t_plain
