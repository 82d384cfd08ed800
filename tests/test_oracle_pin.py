"""Pin the oracle: the CPU port (oracle/port) must reproduce the reference's own
outputs.  Two anchors:
  * the committed golden fixtures, made by running the reference's C sources
    (tests/golden/make_golden.py) -- checked on every machine;
  * the reference build itself (oracle/_ref), where present -- bit-exact checks on
    fresh seeded inputs.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden_cases, load_golden, spectrum_matrix
from lowrankmatrixdecompositioncodes_gb300.capi import ListOmega, SeededOmega
from parity import compare_outputs

GOLDEN_KEYS = sorted(golden_cases())


@pytest.mark.parametrize("key", GOLDEN_KEYS)
def test_port_matches_reference_golden(port, key):
    meta, A, want, omegas = load_golden(key)
    port.set_omega(ListOmega(omegas))
    got = getattr(port, meta["routine"])(A, *meta["args"])
    got = got if isinstance(got, tuple) else (got,)
    assert port.omega_calls() == meta["n_omega"]
    # Same LAPACK calls in the same order: identical on the same OpenBLAS; other
    # OpenBLAS builds (e.g. aarch64) round differently at the 1e-15 level.
    compare_outputs(meta["routine"], got, want, rtol=1e-9)


RANDOM_CASES = [
    ("low_rank_svd_rand_decomp_fixed_rank", (25, 7, 1, 2, 1)),
    ("low_rank_svd_rand_decomp_fixed_rank", (25, 7, 2, 3, 1)),
    ("low_rank_svd_blockrand_decomp_fixed_rank_or_prec", (30, 5, 0.0, 1, 10, 2, 1)),
    ("randQB_pb_new", (10, 0, 1e-3, 1, 1)),
    ("randQB_pb", (10, 4, 1, 1)),
    ("randQB_pb", (8, 5, 2, 2)),
    ("id_rand_decomp_fixed_rank", (25, 5, 2, 1)),
    ("id_two_sided_rand_decomp_fixed_rank", (25, 5, 1, 1)),
    ("cur_rand_decomp_fixed_rank", (25, 5, 2, 1)),
    ("cur_blockrand_decomp_fixed_rank_or_prec", (20, 10, 0.0, 10, 1, 1)),
]


@pytest.mark.parametrize("routine,args", RANDOM_CASES)
@pytest.mark.parametrize("shape", [(150, 110), (110, 150)])
def test_port_bit_exact_with_reference_build(ref, port, routine, args, shape):
    m, n = shape
    A = spectrum_matrix(m, n, 0.97 ** np.arange(min(m, n)), seed=m * 7 + n)
    outs = []
    for lib in (ref, port):
        lib.set_omega(SeededOmega(seed=5))
        o = getattr(lib, routine)(A, *args)
        outs.append(o if isinstance(o, tuple) else (o,))
    compare_outputs(routine, outs[1], outs[0], rtol=0.0)


def test_reference_quirks_are_kept(port):
    """Reference semantics the engine must reproduce (kept in the oracle):
    q means q-1 power rounds in the fixed-rank SVD (one omega request either way),
    vnum==2 returns singular values ascending, S is a dense k x k matrix."""
    A = spectrum_matrix(80, 60, 0.9 ** np.arange(60), seed=3)
    port.set_omega(SeededOmega(1))
    U, S, V = port.low_rank_svd_rand_decomp_fixed_rank(A, 10, 5, 2, 2, 1)
    d = np.diag(S)
    assert S.shape == (10, 10) and np.all(np.diff(d) > 0)
    port.set_omega(SeededOmega(1))
    U, S, V = port.low_rank_svd_rand_decomp_fixed_rank(A, 10, 5, 1, 2, 1)
    assert np.all(np.diff(np.diag(S)) < 0)
    assert port.omega_calls() == 1
    sv = np.linalg.svd(A, compute_uv=False)[:10]
    assert np.allclose(np.diag(S)[:4], sv[:4], rtol=1e-3)


def test_rank_only_pivoted_qr_stops_only_on_exact_zero(ref, port):
    """pivoted_QR_of_specified_rank stops early only on an exactly vanished pivot column
    (rank_revealing_algorithms_intel_mkl.c:1069); the rank-or-precision routine below 1e-10
    (:1250).  A rank-5 matrix plus columns of squared norm ~1e-12: the first stops at k, the
    second after five steps.  The port matches the reference with identical pivots and ranks, and
    factors to 1e-12 (the reference's column norms come from an OpenMP reduction whose order
    depends on the thread count)."""
    g = np.random.default_rng(17)
    B = g.standard_normal((60, 5)) @ g.standard_normal((5, 7))
    A = np.hstack([B, 1e-7 * g.standard_normal((60, 3))])
    outs = {}
    for name, lib in (("ref", ref), ("port", port)):
        outs[name] = (lib.pivoted_QR_of_specified_rank(A, 8), lib.pivoted_QR_of_specified_rank_or_prec(A, 8, 0.0))
    (r1, p1), (r2, p2) = outs["ref"], outs["port"]
    assert r1[3] == 8 and p1[3] == 5
    compare_outputs("pivoted_QR_of_specified_rank", r2, r1, rtol=1e-12)
    compare_outputs("pivoted_QR_of_specified_rank_or_prec", p2, p1, rtol=1e-12)
    # and on a full-rank matrix, rank 12 of 110 columns
    A = spectrum_matrix(150, 110, 0.97 ** np.arange(110), seed=3)
    compare_outputs("pivoted_QR_of_specified_rank", port.pivoted_QR_of_specified_rank(A, 12),
                    ref.pivoted_QR_of_specified_rank(A, 12), rtol=1e-12)


def _old_api(lib):
    L = lib.lib
    for name, n_int in (("randomized_low_rank_svd1", 1), ("randomized_low_rank_svd2", 1),
                        ("randomized_low_rank_svd3", 3), ("randomized_low_rank_svd4", 3)):
        getattr(L, name).argtypes = [lib.PMat] + [lib.Int] * n_int + [C.POINTER(lib.PMat)] * 3
    return L


def test_older_svd_entry_points_are_the_current_routines(ref, port):
    """The identities the engine's randomized_low_rank_svd1..4 rest on, checked on the reference's
    own build: svd1..3 are low_rank_svd_rand_decomp_fixed_rank with fixed parameters (bit for bit),
    svd4 is randQB_pb followed by the eig(B B^T) back end with the pairs ascending (the port's
    QB split, reversed)."""
    L = _old_api(ref)
    A = spectrum_matrix(120, 80, 0.9 ** np.arange(80), seed=1)

    def old(name, *a):
        ref.set_omega(SeededOmega(3))
        M = ref.to_mat(A)
        U, S, V = ref.PMat(), ref.PMat(), ref.PMat()
        getattr(L, name)(M, *a, C.byref(U), C.byref(S), C.byref(V))
        L.matrix_delete(M)
        return ref.from_mat(U), ref.from_mat(S), ref.from_mat(V)

    for name, a_old, a_new in (("randomized_low_rank_svd1", (10,), (10, 0, 2, 1, 1)),
                               ("randomized_low_rank_svd2", (10,), (10, 0, 1, 1, 1)),
                               ("randomized_low_rank_svd3", (10, 3, 2), (10, 0, 1, 3, 2))):
        ref.set_omega(SeededOmega(3))
        want = ref.low_rank_svd_rand_decomp_fixed_rank(A, *a_new)
        assert all(np.array_equal(x, y) for x, y in zip(old(name, *a_old), want)), name
    U4, S4, V4 = old("randomized_low_rank_svd4", 6, 3, 1)
    ref.set_omega(SeededOmega(3))
    Q, B = ref.randQB_pb(A, 6, 3, 1, 1)
    U, S, V = port.low_rank_svd_rand_decomp_fromQB(Q, B)
    assert np.max(np.abs(np.diag(S4) - np.diag(S)[::-1])) < 1e-13
    compare_outputs("low_rank_svd_rand_decomp_fixed_rank", (U4, S4, V4), (U[:, ::-1], S[::-1, ::-1], V[:, ::-1]),
                    rtol=1e-12)
