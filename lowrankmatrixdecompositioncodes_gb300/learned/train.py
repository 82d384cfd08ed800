"""Train the proposal network on the GPU with the engine's own kernels and write the weights.

  python -m lowrankmatrixdecompositioncodes_gb300.learned.dataset --out train20k.npz   # (CPU, once)
  python -m lowrankmatrixdecompositioncodes_gb300.learned.train \\
      --data train20k.npz \\
      --out  lowrankmatrixdecompositioncodes_gb300/learned/proposal_mlp.bin

The last 10% of the (seeded, shuffled) set is held out: it calibrates the safety margin and
reports the validation error (log2 width) printed at the end.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from .. import load_engine
from . import model


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--data", required=True)
    ap.add_argument("--out", required=True)
    ap.add_argument("--epochs", type=int, default=80)
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args()
    d = np.load(a.data)
    F, W, R = d["features"], d["widths"], d["reached"]
    T = model.targets(W)
    n = len(F)
    perm = np.random.default_rng(a.seed).permutation(n)
    nv = n // 10
    va, tr = perm[:nv], perm[nv:]
    eng = load_engine()
    trainer = model.Trainer(eng)
    P, norm = trainer.fit(F[tr], T[tr], R[tr], epochs=a.epochs, seed=a.seed)
    pred = trainer.predict(P, norm, F[va])
    margin = model.calibrate_margin(pred, T[va], R[va])
    model.save(a.out, trainer.dims, P, norm, margin)
    ok = R[va] > 0
    mae = [float(np.mean(np.abs(pred[ok[:, j], j] - T[va][ok[:, j], j]))) for j in range(T.shape[1])]
    cover = [float(np.mean(pred[ok[:, j], j] + margin[j] >= T[va][ok[:, j], j])) for j in range(T.shape[1])]
    print(json.dumps({"train": int(len(tr)), "val": int(nv), "val_mae_log2": mae, "margin_log2": margin.tolist(),
                      "val_coverage_with_margin": cover, "out": a.out}))


if __name__ == "__main__":
    main()
