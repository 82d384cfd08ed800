"""Comparison rules shared by the parity tests.

Outputs of each reference routine, with how two runs of the same algorithm may
legitimately differ:
  'cols'  orthonormal factor: equal up to the sign of each column
  'rows'  factor whose rows pair with a 'cols' factor: equal up to the same signs
  'f'     sign-invariant floating-point output
  'idx'   0-based index vector (stored as doubles): must be identical
  'int'   returned rank: must be identical
"""
from __future__ import annotations

import numpy as np

KINDS = {
    "low_rank_svd_rand_decomp_fixed_rank": ("cols", "f", "cols"),
    "low_rank_svd_blockrand_decomp_fixed_rank_or_prec": ("cols", "f", "cols", "int"),
    "randQB_pb_new": ("cols", "rows", "int"),
    "randQB_pb2": ("cols", "rows", "int"),
    "randQB_pb": ("cols", "rows"),
    "pivotedQR_mkl": ("cols", "rows", "idx"),
    "pivoted_QR_of_specified_rank_or_prec": ("cols", "rows", "idx", "int"),
    "pivoted_QR_of_specified_rank": ("cols", "rows", "idx", "int"),
    "id_decomp_fixed_rank_or_prec": ("idx", "f", "int"),
    "id_rand_decomp_fixed_rank": ("idx", "f"),
    "id_blockrand_decomp_fixed_rank_or_prec": ("idx", "f", "int"),
    "id_two_sided_decomp_fixed_rank_or_prec": ("idx", "idx", "f", "f", "int"),
    "id_two_sided_rand_decomp_fixed_rank": ("idx", "idx", "f", "f"),
    "id_two_sided_blockrand_decomp_fixed_rank_or_prec": ("idx", "idx", "f", "f", "int"),
    "cur_decomp_fixed_rank_or_prec": ("f", "f", "f", "int"),
    "cur_rand_decomp_fixed_rank": ("f", "f", "f"),
    "cur_blockrand_decomp_fixed_rank_or_prec": ("f", "f", "f", "int"),
    "low_rank_svd_rand_decomp_fromQB": ("cols", "f", "cols"),
    "id_rand_decomp_fromQB": ("idx", "f"),
}


def col_signs(X, Y):
    """Signs s with X[:, j] ~ s[j] * Y[:, j], read at each column's largest entry of Y."""
    if X.size == 0:
        return np.ones(X.shape[1])
    piv = np.argmax(np.abs(Y), axis=0)
    cols = np.arange(X.shape[1])
    s = np.sign(X[piv, cols]) * np.sign(Y[piv, cols])
    s[s == 0] = 1.0
    return s


def rel_err(X, Y):
    X = np.asarray(X, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    scale = max(np.max(np.abs(Y)) if Y.size else 0.0, 1e-300)
    return float(np.max(np.abs(X - Y)) / scale) if X.size else 0.0


def compare_outputs(routine, got, want, rtol):
    """Return a list of (index, kind, error) and raise AssertionError on mismatch."""
    kinds = KINDS[routine]
    assert len(got) == len(want) == len(kinds), (len(got), len(want), kinds)
    signs = None
    report = []
    for i, (kind, g, w) in enumerate(zip(kinds, got, want)):
        if kind == "int":
            assert int(g) == int(w), f"output {i}: rank {g} != {w}"
            report.append((i, kind, 0.0))
            continue
        g = np.asarray(g, dtype=np.float64)
        w = np.asarray(w, dtype=np.float64)
        assert g.shape == w.shape, f"output {i}: shape {g.shape} != {w.shape}"
        if kind == "idx":
            assert np.array_equal(g, w), f"output {i}: index sets differ at {np.nonzero(g != w)[0][:10]}"
            report.append((i, kind, 0.0))
            continue
        if kind == "cols":
            s = col_signs(g, w)
            if signs is None:
                signs = s
            g = g * s[None, :]
        elif kind == "rows":
            g = g * signs[: g.shape[0], None]
        e = rel_err(g, w)
        report.append((i, kind, e))
        assert e <= rtol, f"output {i} ({kind}): relative error {e:.3e} > {rtol:.1e}"
    return report
