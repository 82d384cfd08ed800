"""Generate the float-data golden fixtures in tests/golden/f32/ by running the REFERENCE's own
oneAPI-variant code (oneapi_code/, float data, int64_t dimensions), compiled unchanged into
oracle/_ref/librsvd_ref_f32.so by ``make -C oracle ref``.

The inputs are the float32 roundings of the double fixtures' matrices (tests/golden/*__A.npz);
every Gaussian test matrix is served from a recorded seeded provider and stored with the outputs,
so a float-data implementation can be replayed on exactly the reference's inputs anywhere.  The
QB-split cases take the Q and B of the reference's own randQB_pb2 run as their inputs.

Run here, where the reference tree exists:
    make -C oracle ref && python tests/golden/make_golden_f32.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "f32")
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lowrankmatrixdecompositioncodes_gb300.capi import RsvdLibrary, SeededOmega  # noqa: E402

# (case name, routine of the oneAPI ABI, positional arguments after the matrix); a TOL given as
# ("rel", x) is x * ||A||_F of the case's matrix
CASES = [
    ("svd_v1_q2", "low_rank_svd_rand_decomp_fixed_rank", (12, 4, 1, 2, 1)),
    ("svd_v2_q2", "low_rank_svd_rand_decomp_fixed_rank", (12, 4, 2, 2, 1)),
    ("qb2_rank", "randQB_pb2", (6, 4, 0.0, 1, 1)),
    ("qb2_tol", "randQB_pb2", (6, 0, ("rel", 1e-3), 1, 1)),
    ("qb_pb", "randQB_pb", (6, 4, 1, 1)),
    ("id_rand", "id_rand_decomp_fixed_rank", (12, 4, 2, 1)),
    ("pivqr_full", "pivotedQR_mkl", ()),
]
SPLIT_CASES = [
    ("fromqb_svd", "low_rank_svd_rand_decomp_fromQB"),
    ("fromqb_id", "id_rand_decomp_fromQB"),
]


def main():
    lib_path = os.path.join(ROOT, "oracle", "_ref", "librsvd_ref_f32.so")
    if not os.path.exists(lib_path):
        raise SystemExit("build the reference first: make -C oracle ref")
    ref = RsvdLibrary(lib_path, real32=True)
    os.makedirs(OUT, exist_ok=True)
    index = {}
    for mname in ("tall", "wide"):
        A = np.load(os.path.join(HERE, f"{mname}__A.npz"))["A"].astype(np.float32)
        np.savez_compressed(os.path.join(OUT, f"{mname}__A.npz"), A=A)
        fro = float(np.linalg.norm(A.astype(np.float64)))
        qb = None
        for cname, routine, args in CASES:
            args = tuple(float(np.float32(a[1] * fro)) if isinstance(a, tuple) else a for a in args)
            om = SeededOmega(seed=5000 + len(index))
            om.record = True
            ref.set_omega(om)
            out = getattr(ref, routine)(A, *args)
            out = out if isinstance(out, tuple) else (out,)
            if cname == "qb2_rank":
                qb = (out[0], out[1])
            key = f"{mname}__{cname}"
            payload = {f"out{i}": np.asarray(o) for i, o in enumerate(out)}
            payload.update({f"omega{i}": w for i, w in enumerate(om.served)})
            np.savez_compressed(os.path.join(OUT, f"{key}.npz"), **payload)
            index[key] = {"routine": routine, "args": list(args), "n_out": len(out), "matrix": f"{mname}__A.npz",
                          "n_omega": len(om.served), "shape": list(A.shape)}
        for cname, routine in SPLIT_CASES:
            out = getattr(ref, routine)(*qb)
            key = f"{mname}__{cname}"
            payload = {"Q": qb[0], "B": qb[1]}
            payload.update({f"out{i}": np.asarray(o) for i, o in enumerate(out)})
            np.savez_compressed(os.path.join(OUT, f"{key}.npz"), **payload)
            index[key] = {"routine": routine, "args": [], "n_out": len(out), "matrix": None, "n_omega": 0,
                          "shape": list(A.shape)}
    with open(os.path.join(OUT, "index.json"), "w") as f:
        json.dump(index, f, indent=1, sort_keys=True)
    print(f"wrote {len(index)} fixtures")


if __name__ == "__main__":
    main()
