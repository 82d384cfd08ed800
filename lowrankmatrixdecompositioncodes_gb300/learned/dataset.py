"""Training set for the learned rank / power-count proposal.

Each sample is a generated spectrum s (length r = min(m, n)), a tolerance TOL and the
outcome of runs of the method itself on it:

  features : the 32 R-diagonal magnitudes of a 32-column probe sketch Y0 = A Omega0 (relative
             to ||A||_F, log10), the energy the probe leaves, log10 max(1 - sum_j R_jj^2 /
             ||A||_F^2, 1e-5) (floored where FP32 rounding would blur it), log10 r,
             log10(m / n) and log10 TOL.
  labels   : for q = 1 and q = 2 power iterations, the smallest sketch width l (a multiple
             of 32) at which the single-shot randomized range finder with l Gaussian
             columns and q power iterations reaches ||A - Q Q^T A||_F <= TOL ||A||_F, and
             whether that width was reached within the cap.

Why the runs use A = diag(s): for a Gaussian test matrix Omega, U diag(s) V^T Omega has the
distribution of U diag(s) Omega, so the probe's R factor and the range finder's residual
have exactly the distribution they have for any matrix with singular values s and Haar
factors U, V.  The method is therefore run on the diagonal operator, and only its r x l
sketch is formed.

Residual of the width-l prefix: with Q from a Householder QR of Y = diag(s^(2q+1)) Omega,
||A - Q_l Q_l^T A||_F^2 = ||s||^2 - sum_{j<l} sum_i s_i^2 Q_ij^2 (FP64; for TOL >= 1e-6 the
cancellation leaves >= 4 significant digits).  Rows with s_i^(2q+1) below 1e-18 of the
largest do not enter Y (their rows of Q vanish to working precision), but their energy stays
in ||s||^2.

Run `python -m lowrankmatrixdecompositioncodes_gb300.learned.dataset --out FILE` to build the
set (multiprocessing, seeded; about an hour on 8 cores for 20k samples).
"""
from __future__ import annotations

import argparse
import os
import time

import numpy as np

PROBE = 32
QS = (1, 2)
L_CAP = 3072
N_FEATURES = PROBE + 4


def spectrum(rng: np.random.Generator, r: int) -> tuple[np.ndarray, str]:
    """A seeded spectrum of length r: exponential, power-law (exponent 0.5-3), step plus
    noise, or a mixture of two of them; normalised to s_1 = 1 and sorted descending."""
    i = np.arange(1, r + 1, dtype=np.float64)
    kind = rng.choice(["exp", "pow", "step", "mix"], p=[0.35, 0.25, 0.2, 0.2])

    def one(k):
        if k == "exp":
            tau = float(np.exp(rng.uniform(np.log(5.0), np.log(300.0))))
            return np.exp(-(i - 1) / tau)
        if k == "pow":
            return i ** (-rng.uniform(0.5, 3.0))
        rank = int(np.exp(rng.uniform(np.log(8.0), np.log(min(2000.0, r / 2)))))
        floor = 10.0 ** rng.uniform(-8.0, -3.0)
        s = floor * np.exp(-(i - 1) / rng.uniform(50.0, 2000.0))
        s[:rank] += np.exp(-(i[:rank] - 1) / rng.uniform(rank / 4.0, 4.0 * rank))
        s *= 1.0 + 0.05 * rng.standard_normal(r)
        return np.abs(s)

    if kind == "mix":
        a, b = rng.choice(["exp", "pow", "step"], size=2, replace=True)
        w = 10.0 ** rng.uniform(-4.0, 0.0)
        s = one(a) + w * one(b)
    else:
        s = one(kind)
    s = np.sort(s)[::-1]
    return s / s[0], str(kind)


def probe_features(s: np.ndarray, m: int, n: int, tol: float, rng: np.random.Generator) -> np.ndarray:
    """R-diagonal features of the 32-column probe sketch of diag(s) (the same quantities
    the engine computes from A Omega0 for a dense A)."""
    r = s.size
    Y = s[:, None] * rng.standard_normal((r, PROBE))
    R = np.linalg.qr(Y, mode="r")
    d = np.abs(np.diag(R))
    fro = float(np.sqrt(np.sum(s * s)))
    return feature_vector(d, fro, m, n, tol)


def feature_vector(rdiag: np.ndarray, fro: float, m: int, n: int, tol: float) -> np.ndarray:
    """The model's input from the probe's R-diagonal (length 32), ||A||_F, the shape and TOL."""
    rel = np.maximum(np.asarray(rdiag, dtype=np.float64) / fro, 1e-30)
    f = np.empty(N_FEATURES, dtype=np.float64)
    f[:PROBE] = np.log10(rel)
    f[PROBE] = np.log10(max(1.0 - float(np.sum(rel * rel)), 1e-5))
    f[PROBE + 1] = np.log10(min(m, n))
    f[PROBE + 2] = np.log10(m / n)
    f[PROBE + 3] = np.log10(tol)
    return f


def needed_width(s: np.ndarray, tol: float, q: int, rng: np.random.Generator) -> tuple[int, bool]:
    """Smallest multiple of 32 (<= min(r, L_CAP)) at which the single-shot range finder with q
    power iterations reaches the tolerance on diag(s); (cap, False) if it does not."""
    r = s.size
    tot = float(np.sum(s * s))
    tail = np.sqrt(np.maximum(tot - np.cumsum(s * s), 0.0) / tot)        # optimal rank-k error
    k_opt = int(np.searchsorted(-tail, -tol)) + 1                          # first k with tail <= tol
    cap = min(r, L_CAP)
    t = s ** (2 * q + 1)
    keep = t >= 1e-18 * t[0]
    for grow in (1.15, 1.6):                    # first try a width near k_opt, then a wider one
        L = int(min(cap, 32 * int(np.ceil((grow * k_opt + 64) / 32.0))))
        ne = min(max(int(np.count_nonzero(keep)), L), r)
        Y = t[:ne, None] * rng.standard_normal((ne, L))
        Q = np.linalg.qr(Y, mode="reduced")[0]
        energy = (s[:ne] ** 2) @ (Q * Q)                                   # captured per column
        res = np.sqrt(np.maximum(tot - np.cumsum(energy), 0.0) / tot)
        ok = np.nonzero(res <= tol)[0]
        if ok.size:
            l = int(ok[0]) + 1
            return min(cap, 32 * int(np.ceil(l / 32.0))), True
        if L >= cap:
            break
    return cap, False


def sample(seed: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    rng = np.random.default_rng(seed)
    m = int(rng.integers(1024, 8193))
    n = int(rng.integers(1024, 8193))
    r = min(m, n)
    s, _ = spectrum(rng, r)
    tol = float(10.0 ** rng.uniform(-6.0, -2.0))
    f = probe_features(s, m, n, tol, rng)
    widths = np.zeros(len(QS), dtype=np.float64)
    reached = np.zeros(len(QS), dtype=np.float64)
    for j, q in enumerate(QS):
        w, ok = needed_width(s, tol, q, rng)
        widths[j], reached[j] = w, float(ok)
    return f, widths, reached


def features_only(seed: int) -> np.ndarray:
    """The feature vector of sample(seed), without the label runs (the probe draws its test
    matrix before the labels do, so the stream is the same)."""
    rng = np.random.default_rng(seed)
    m = int(rng.integers(1024, 8193))
    n = int(rng.integers(1024, 8193))
    s, _ = spectrum(rng, min(m, n))
    tol = float(10.0 ** rng.uniform(-6.0, -2.0))
    return probe_features(s, m, n, tol, rng)


def _work(args):
    lo, hi, base = args
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    out = [sample(base + i) for i in range(lo, hi)]
    return lo, out


def build(count: int, base_seed: int, procs: int) -> dict:
    import multiprocessing as mp
    chunks = [(i, min(count, i + 64), base_seed) for i in range(0, count, 64)]
    F = np.zeros((count, N_FEATURES))
    W = np.zeros((count, len(QS)))
    OK = np.zeros((count, len(QS)))
    ctx = mp.get_context("spawn")
    t0 = time.time()
    with ctx.Pool(procs) as pool:
        done = 0
        for lo, out in pool.imap_unordered(_work, chunks):
            for j, (f, w, ok) in enumerate(out):
                F[lo + j], W[lo + j], OK[lo + j] = f, w, ok
            done += len(out)
            if done % 2048 < 64:
                print(f"{done}/{count} samples, {time.time() - t0:.0f} s", flush=True)
    return {"features": F.astype(np.float32), "widths": W.astype(np.float32), "reached": OK.astype(np.float32),
            "qs": np.array(QS, dtype=np.int32), "base_seed": np.int64(base_seed), "l_cap": np.int32(L_CAP)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--count", type=int, default=20000)
    ap.add_argument("--seed", type=int, default=1_000_000)
    ap.add_argument("--procs", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--refeature", help="recompute the features of an existing set (labels kept)")
    a = ap.parse_args()
    if a.refeature:
        d = dict(np.load(a.refeature))
        base = int(d["base_seed"])
        d["features"] = np.stack([features_only(base + i) for i in range(len(d["features"]))]).astype(np.float32)
        np.savez_compressed(a.out, **d)
        print("refeatured", a.out)
        return
    d = build(a.count, a.seed, a.procs)
    np.savez_compressed(a.out, **d)
    print("wrote", a.out, {k: v.shape for k, v in d.items() if hasattr(v, "shape")})


if __name__ == "__main__":
    main()
