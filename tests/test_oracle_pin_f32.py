"""Pin the float-data variant against the double one, where the reference tree is present.

oracle/_ref/librsvd_ref_f32.so is the oneAPI variant's own sources (oneapi_code/, float data,
int64_t dimensions) compiled unchanged; oracle/_ref/librsvd_ref.so the MKL variant's.  On the same
float-representable matrix and the same test matrices they must agree to single-precision
rounding: the premise of librsvdpack_f32.so, which serves the oneAPI ABI with the algorithms of
the MKL variant.  The oneAPI variant's QB split (low_rank_svd_rand_decomp_fromQB,
id_rand_decomp_fromQB, rank_revealing_algorithms_one_api.c:244,421), which the MKL variant does
not have, is checked against the oracle port's FP64 restatement of it.
"""
import os

import numpy as np
import pytest

from conftest import ROOT, spectrum_matrix
from lowrankmatrixdecompositioncodes_gb300.capi import RsvdLibrary, SeededOmega
from parity import col_signs

REF_F32_SO = os.path.join(ROOT, "oracle", "_ref", "librsvd_ref_f32.so")


@pytest.fixture(scope="module")
def ref_f32():
    if not os.path.exists(REF_F32_SO):
        pytest.skip("oneAPI reference build (oracle/_ref) not present on this machine")
    return RsvdLibrary(REF_F32_SO, real32=True)


def _matrix(m, n, decay, seed):
    return spectrum_matrix(m, n, decay ** np.arange(min(m, n)), seed).astype(np.float32)


def _run(lib, name, A, *args, seed=7):
    lib.set_omega(SeededOmega(seed))
    return getattr(lib, name)(A, *args)


def _close_cols(X32, X64, tol):
    X32 = np.asarray(X32, dtype=np.float64)
    s = col_signs(X32, X64)
    assert np.max(np.abs(X32 * s - X64)) <= tol * max(np.abs(X64).max(), 1e-30)


@pytest.mark.parametrize("vnum", [1, 2])
def test_fixed_rank_svd_agrees(ref, ref_f32, vnum):
    A = _matrix(300, 200, 0.9, 3)
    U1, S1, V1 = _run(ref, "low_rank_svd_rand_decomp_fixed_rank", A, 20, 8, vnum, 2, 1)
    U2, S2, V2 = _run(ref_f32, "low_rank_svd_rand_decomp_fixed_rank", A, 20, 8, vnum, 2, 1)
    s1, s2 = np.diag(S1), np.diag(S2).astype(np.float64)
    assert np.max(np.abs(s2 - s1) / s1) < 1e-4
    _close_cols(U2, U1, 1e-3)
    _close_cols(V2, V1, 1e-3)


def test_blocked_qb_variants_agree(ref, ref_f32):
    A = _matrix(256, 192, 0.9, 5)
    # randQB_pb2 (oneAPI) is randQB_pb_new (MKL): rank mode and TOL mode
    for args in ((16, 4, 0.0, 1, 1), (16, 0, 1e-3 * float(np.linalg.norm(A)), 1, 1)):
        Q1, B1, f1 = _run(ref, "randQB_pb_new", A, *args)
        Q2, B2, f2 = _run(ref_f32, "randQB_pb2", A, *args)
        assert f1 == f2 > 0
        assert np.linalg.norm(Q2.astype(np.float64) @ B2 - Q1 @ B1) < 1e-4 * np.linalg.norm(A)
    # randQB_pb: every block after the first re-orthogonalised, in both variants
    Q1, B1 = _run(ref, "randQB_pb", A, 16, 4, 1, 1)
    Q2, B2 = _run(ref_f32, "randQB_pb", A, 16, 4, 1, 1)
    assert Q2.shape == Q1.shape == (256, 64)
    assert np.linalg.norm(Q2.astype(np.float64) @ B2 - Q1 @ B1) < 1e-4 * np.linalg.norm(A)


def test_id_and_pivoted_qr_agree(ref, ref_f32):
    A = _matrix(200, 300, 0.85, 9)
    I1, T1 = _run(ref, "id_rand_decomp_fixed_rank", A, 15, 5, 2, 1)
    I2, T2 = _run(ref_f32, "id_rand_decomp_fixed_rank", A, 15, 5, 2, 1)
    assert np.array_equal(I1, I2.astype(np.float64))
    assert np.max(np.abs(T2 - T1)) < 1e-3 * np.abs(T1).max()
    Q1, R1, J1 = ref.pivotedQR_mkl(A[:, :40])
    Q2, R2, J2 = ref_f32.pivotedQR_mkl(A[:, :40])
    assert np.array_equal(J1, J2.astype(np.float64))
    _close_cols(Q2, Q1, 1e-3)


def test_qb_split_matches_the_port(port, ref_f32):
    """The oneAPI QB split against the port's FP64 restatement of it, on the same Q and B."""
    A = _matrix(240, 160, 0.9, 11).astype(np.float64)
    rng = np.random.default_rng(2)
    Q, _ = np.linalg.qr(A @ rng.standard_normal((160, 24)))
    Q = Q.astype(np.float32).astype(np.float64)
    B = (Q.T @ A).astype(np.float32).astype(np.float64)
    U1, S1, V1 = port.low_rank_svd_rand_decomp_fromQB(Q, B)
    U2, S2, V2 = ref_f32.low_rank_svd_rand_decomp_fromQB(Q, B)
    s1, s2 = np.diag(S1), np.diag(S2).astype(np.float64)
    top = s1 > 1e-3 * s1[0]                     # float's eig(B B^T) resolves sigma^2 to ~1e-7
    assert np.max(np.abs(s2[top] - s1[top]) / s1[top]) < 1e-4
    _close_cols(U2[:, top], U1[:, top], 1e-3)
    I1, T1 = port.id_rand_decomp_fromQB(Q, B)
    I2, T2 = ref_f32.id_rand_decomp_fromQB(Q, B)
    assert np.array_equal(I1, I2.astype(np.float64))
    assert np.max(np.abs(T2 - T1)) < 1e-3 * np.abs(T1).max()


# ---------------------------------------------------------------- float golden fixtures
GOLDEN_F32 = os.path.join(ROOT, "tests", "golden", "f32")


def _golden_f32():
    import json
    with open(os.path.join(GOLDEN_F32, "index.json")) as f:
        return json.load(f)


def _load_f32(key, meta):
    z = np.load(os.path.join(GOLDEN_F32, key + ".npz"))
    outs = [z[f"out{i}"] for i in range(meta["n_out"])]
    if meta["matrix"] is None:
        return (z["Q"], z["B"]), outs, []
    A = np.load(os.path.join(GOLDEN_F32, meta["matrix"]))["A"]
    return (A,), outs, [z[f"omega{i}"] for i in range(meta["n_omega"])]


F32_KEYS = sorted(_golden_f32())
# the MKL-variant name of each oneAPI routine
MKL_NAME = {"randQB_pb2": "randQB_pb_new"}


@pytest.mark.parametrize("key", F32_KEYS)
def test_oneapi_reference_reproduces_float_golden(ref_f32, key):
    from lowrankmatrixdecompositioncodes_gb300.capi import ListOmega
    from parity import compare_outputs
    meta = _golden_f32()[key]
    inputs, want, omegas = _load_f32(key, meta)
    ref_f32.set_omega(ListOmega(omegas))
    got = getattr(ref_f32, meta["routine"])(*inputs, *meta["args"])
    got = got if isinstance(got, tuple) else (got,)
    compare_outputs(meta["routine"].replace("randQB_pb2", "randQB_pb_new"), got, want, rtol=1e-5)


@pytest.mark.parametrize("key", F32_KEYS)
def test_port_matches_float_golden_to_single_precision(port, key):
    """On every machine: the oracle port (the MKL variant's algorithms, FP64) replayed on the float
    fixtures' inputs and test matrices gives the oneAPI reference's float outputs to single-precision
    rounding -- identical pivots and ranks, factors to 2e-3 of each output's largest entry."""
    from lowrankmatrixdecompositioncodes_gb300.capi import ListOmega
    from parity import compare_outputs
    meta = _golden_f32()[key]
    inputs, want, omegas = _load_f32(key, meta)
    routine = MKL_NAME.get(meta["routine"], meta["routine"])
    port.set_omega(ListOmega(omegas))
    got = getattr(port, routine)(*[x.astype(np.float64) for x in inputs], *meta["args"])
    got = got if isinstance(got, tuple) else (got,)
    want = [np.asarray(w, dtype=np.float64) for w in want]
    if routine == "pivotedQR_mkl":
        # a full factorisation of a matrix whose spectrum spans 1e-6: in single precision the
        # reflectors after |R_ii| falls below ~1e-3 |R_00| act on rounding noise, so the leading
        # part (pivots, Q columns, R rows) is what the two precisions share
        Q, R, I = got
        r = int(np.sum(np.abs(np.diag(R)) > 1e-3 * abs(R[0, 0])))
        got = (Q[:, :r], R[:r, :], I[:r])
        want = [want[0][:, :r], want[1][:r, :], want[2][:r]]
    compare_outputs(routine, got, want, rtol=2e-3)
