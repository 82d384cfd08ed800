"""Generate the golden fixtures in tests/golden/ by running the REFERENCE's own code.

The reference ships no tests, fixtures or golden vectors, and its Gaussian test
matrices are time-seeded, so nothing of it is reproducible as shipped.  This
script pins it: it runs the reference's C sources (compiled unchanged into
oracle/_ref/librsvd_ref.so by ``make -C oracle ref``) on small seeded matrices,
serving every Gaussian test matrix from a recorded seeded provider, and stores
inputs, the served test matrices and all outputs as .npz files.

Run here, where the reference tree exists:
    make -C oracle ref && python tests/golden/make_golden.py
The fixtures are then checked in; tests read them on any machine.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lowrankmatrixdecompositioncodes_gb300.capi import RsvdLibrary, SeededOmega  # noqa: E402


def spectrum_matrix(m, n, s, seed):
    """A = U diag(s) V^T with U, V the Q factors of seeded Gaussian matrices."""
    g = np.random.default_rng(seed)
    r = min(m, n)
    U, _ = np.linalg.qr(g.standard_normal((m, r)))
    V, _ = np.linalg.qr(g.standard_normal((n, r)))
    return (U * s[:r]) @ V.T


# (case name, reference routine, positional arguments after the matrix)
CASES = [
    ("svd_v1_q2", "low_rank_svd_rand_decomp_fixed_rank", (12, 4, 1, 2, 1)),
    ("svd_v1_q3_s2", "low_rank_svd_rand_decomp_fixed_rank", (12, 4, 1, 3, 2)),
    ("svd_v2_q2", "low_rank_svd_rand_decomp_fixed_rank", (12, 4, 2, 2, 1)),
    ("svd_v1_q1", "low_rank_svd_rand_decomp_fixed_rank", (10, 6, 1, 1, 1)),
    ("blk_svd_rank", "low_rank_svd_blockrand_decomp_fixed_rank_or_prec", (16, 4, 0.0, 1, 8, 1, 1)),
    ("blk_svd_rank_v2", "low_rank_svd_blockrand_decomp_fixed_rank_or_prec", (16, 4, 0.0, 2, 8, 2, 1)),
    ("blk_svd_tol", "low_rank_svd_blockrand_decomp_fixed_rank_or_prec", (0, 4, 1e-3, 1, 8, 1, 1)),
    ("qb_rank", "randQB_pb_new", (6, 4, 0.0, 1, 1)),
    ("qb_rank_q2s2", "randQB_pb_new", (6, 3, 0.0, 2, 2)),
    ("qb_tol", "randQB_pb_new", (6, 0, 1e-4, 1, 1)),
    ("pivqr_full", "pivotedQR_mkl", ()),
    ("pivqr_rank", "pivoted_QR_of_specified_rank_or_prec", (10, 0.0)),
    ("pivqr_tol", "pivoted_QR_of_specified_rank_or_prec", (0, 1e-5)),
    ("id_det", "id_decomp_fixed_rank_or_prec", (10, 0.0)),
    ("id_rand", "id_rand_decomp_fixed_rank", (12, 4, 2, 1)),
    ("id_rand_q1s2", "id_rand_decomp_fixed_rank", (12, 4, 1, 2)),
    ("id_blk", "id_blockrand_decomp_fixed_rank_or_prec", (12, 4, 0.0, 8, 1, 1)),
    ("id2_det", "id_two_sided_decomp_fixed_rank_or_prec", (10, 0.0)),
    ("id2_rand", "id_two_sided_rand_decomp_fixed_rank", (12, 4, 2, 1)),
    ("id2_blk", "id_two_sided_blockrand_decomp_fixed_rank_or_prec", (12, 4, 0.0, 8, 1, 1)),
    ("cur_det", "cur_decomp_fixed_rank_or_prec", (10, 0.0)),
    ("cur_rand", "cur_rand_decomp_fixed_rank", (12, 4, 2, 1)),
    ("cur_blk", "cur_blockrand_decomp_fixed_rank_or_prec", (12, 4, 0.0, 8, 1, 1)),
]

MATRICES = {
    # tall, spectrum 10^(-6(i-1)/(r-1)) as in the plain fixed-rank workload
    "tall": (96, 64, lambda r: 10.0 ** (-6.0 * np.arange(r) / (r - 1)), 11),
    # wide, power-law spectrum i^-2 as in the ID/CUR workload
    "wide": (64, 96, lambda r: (1.0 + np.arange(r)) ** -2.0, 12),
}


def main():
    lib_path = os.path.join(ROOT, "oracle", "_ref", "librsvd_ref.so")
    if not os.path.exists(lib_path):
        raise SystemExit("build the reference first: make -C oracle ref")
    ref = RsvdLibrary(lib_path)
    index = {}
    for mname, (m, n, spec, seed) in MATRICES.items():
        A = spectrum_matrix(m, n, spec(min(m, n)), seed)
        np.savez_compressed(os.path.join(HERE, f"{mname}__A.npz"), A=A)
        for cname, routine, args in CASES:
            om = SeededOmega(seed=1000 + len(index))
            om.record = True
            ref.set_omega(om)
            out = getattr(ref, routine)(A, *args)
            out = out if isinstance(out, tuple) else (out,)
            key = f"{mname}__{cname}"
            payload = {"args": np.array(args, dtype=np.float64)}
            for i, o in enumerate(out):
                payload[f"out{i}"] = np.asarray(o)
            for i, w in enumerate(om.served):
                payload[f"omega{i}"] = w
            np.savez_compressed(os.path.join(HERE, f"{key}.npz"), **payload)
            index[key] = {"routine": routine, "args": list(args), "n_out": len(out),
                          "matrix": f"{mname}__A.npz",
                          "n_omega": len(om.served), "shape": [m, n]}
    with open(os.path.join(HERE, "index.json"), "w") as f:
        json.dump(index, f, indent=1, sort_keys=True)
    print(f"wrote {len(index)} fixtures")


if __name__ == "__main__":
    main()
