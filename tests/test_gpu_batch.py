"""Batched fixed-rank rSVD (rsvdpack_batch_plan_*), through the C ABI.

Every item's test matrix is a Philox4x32-10 stream (seed, item index); the test rebuilds it
on the host and hands the same matrix to the CPU oracle, so each batch item is compared
with the reference algorithm run on the same sketch: singular values, factors up to sign
and the residual, within FP32 tolerances.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import spectrum_matrix
from lowrankmatrixdecompositioncodes_gb300.capi import ListOmega

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF


def philox_gaussians(count, seed, offset):
    """Host restatement of the engine's Philox4x32-10 + Box-Muller stream (float32 values)."""
    groups = (count + 3) // 4
    g = np.arange(groups, dtype=np.uint64)
    x = g & MASK
    y = g >> 32
    z = np.full(groups, offset & MASK, dtype=np.uint64)
    w = np.full(groups, (offset >> 32) & MASK, dtype=np.uint64)
    k0, k1 = seed & MASK, (seed >> 32) & MASK
    for _ in range(10):
        p0 = x * np.uint64(M0)
        p1 = z * np.uint64(M1)
        hi0, lo0 = p0 >> np.uint64(32), p0 & np.uint64(MASK)
        hi1, lo1 = p1 >> np.uint64(32), p1 & np.uint64(MASK)
        x, y, z, w = hi1 ^ y ^ np.uint64(k0), lo1, hi0 ^ w ^ np.uint64(k1), lo0
        k0 = (k0 + W0) & MASK
        k1 = (k1 + W1) & MASK
    u = np.stack([x, y, z, w], axis=1).astype(np.float32)
    scale = np.float32(2.3283064365386963e-10)
    out = np.empty((groups, 4), dtype=np.float64)
    for h in range(2):
        u1 = ((u[:, 2 * h] + np.float32(1.0)) * scale).astype(np.float64)
        u2 = (u[:, 2 * h + 1] * scale).astype(np.float64)
        rad = np.sqrt(-2.0 * np.log(u1))
        out[:, 2 * h] = rad * np.cos(2 * np.pi * u2)
        out[:, 2 * h + 1] = rad * np.sin(2 * np.pi * u2)
    return out.ravel()[:count].astype(np.float32)


def _bind(L):
    L.rsvdpack_batch_plan_create.restype = C.c_void_p
    L.rsvdpack_batch_plan_create.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_ulonglong]
    L.rsvdpack_batch_plan_execute.restype = C.c_int
    L.rsvdpack_batch_plan_execute.argtypes = [C.c_void_p]
    L.rsvdpack_batch_plan_destroy.argtypes = [C.c_void_p]
    L.rsvdpack_batch_plan_info.restype = C.c_int
    L.rsvdpack_batch_plan_info.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                           C.POINTER(C.c_double)]


def plan_info(L, plan):
    lp, cu, tuned, ms = C.c_int(0), C.c_int(0), C.c_int(0), C.c_double(0)
    assert L.rsvdpack_batch_plan_info(plan, C.byref(lp), C.byref(cu), C.byref(tuned), C.byref(ms)) == 0
    return lp.value, cu.value, tuned.value, ms.value


def run_batch(engine, mats, ks, p, q, seed, info=None):
    L = engine.lib
    _bind(L)
    cnt = len(mats)
    dA, dU, dV, dS = [], [], [], []
    for A, k in zip(mats, ks):
        m, n = A.shape
        dA.append(torch.from_numpy(np.asfortranarray(A, dtype=np.float32).T.copy()).cuda())
        dU.append(torch.zeros(k, m, device="cuda", dtype=torch.float32))
        dV.append(torch.zeros(k, n, device="cuda", dtype=torch.float32))
        dS.append(torch.zeros(k, device="cuda", dtype=torch.float64))
    arr = lambda vals, t: (t * cnt)(*vals)
    m = arr([A.shape[0] for A in mats], C.c_int)
    n = arr([A.shape[1] for A in mats], C.c_int)
    kk = arr(ks, C.c_int)
    ptr = lambda ts: (C.c_void_p * cnt)(*[t.data_ptr() for t in ts])
    lda = arr([A.shape[0] for A in mats], C.c_longlong)
    ldv = arr([A.shape[1] for A in mats], C.c_longlong)
    torch.cuda.synchronize()
    plan = L.rsvdpack_batch_plan_create(cnt, m, n, kk, p, q, 1, ptr(dA), lda, ptr(dU), lda, ptr(dS), ptr(dV), ldv,
                                        seed)
    assert plan, engine.last_error()
    if info is not None:
        info.append(plan_info(L, plan))
    try:
        for _ in range(2):                      # the captured graph replays
            rc = L.rsvdpack_batch_plan_execute(plan)
            assert rc == 0, engine.last_error()
    finally:
        L.rsvdpack_batch_plan_destroy(plan)
    return ([u.cpu().numpy().T for u in dU], [s.cpu().numpy() for s in dS], [v.cpu().numpy().T for v in dV])


@pytest.mark.parametrize("q", [1, 2])
def test_batch_matches_oracle_on_the_same_sketches(engine, port, q):
    g = np.random.default_rng(44 + q)
    mats, ks = [], []
    for i in range(24):
        m = int(g.integers(64, 700))
        n = int(g.integers(32, 400))
        A = spectrum_matrix(m, n, 0.9 ** np.arange(min(m, n)), seed=1000 + i)
        mats.append(A.astype(np.float32).astype(np.float64))
        ks.append(max(1, min(m, n) // 8))
    p, seed = 8, 0x1234ABCD
    Us, Ss, Vs = run_batch(engine, mats, ks, p, q, seed)
    for i, (A, k) in enumerate(zip(mats, ks)):
        m, n = A.shape
        om = philox_gaussians(n * (k + p), seed, i)
        port.set_omega(ListOmega([om]))
        Uo, So, Vo = port.low_rank_svd_rand_decomp_fixed_rank(A, k, p, 1, q, 1)
        so = np.diag(So)
        assert np.max(np.abs(Ss[i] - so) / so[0]) < 2e-4, (i, m, n, k)
        res_b = np.linalg.norm(A - (Us[i] * Ss[i]) @ Vs[i].T) / np.linalg.norm(A)
        res_o = np.linalg.norm(A - (Uo * so) @ Vo.T) / np.linalg.norm(A)
        assert abs(res_b - res_o) <= 1e-4 * max(res_o, 1e-3), (i, res_b, res_o)
        assert np.max(np.abs(Us[i].T @ Us[i] - np.eye(k))) < 1e-3
        assert np.max(np.abs(Vs[i].T @ Vs[i] - np.eye(k))) < 1e-3


def test_batch_rejects_oversized_items(engine):
    L = engine.lib
    _bind(L)
    one = (C.c_int * 1)
    null = (C.c_void_p * 1)(0)
    lds = (C.c_longlong * 1)(100)
    plan = L.rsvdpack_batch_plan_create(1, one(100), one(100), one(80), 8, 1, 1, null, lds, null, lds, null, null,
                                        lds, 1)
    assert not plan
    code, msg = engine.last_error()
    assert code == 1 and "72" in msg


def test_batch_autotuner_chooses_and_records(engine, port):
    """Plan creation times the kernel's configurations (lanes per Jacobi pair x column-group
    offset) on a sample of the batch and records the fastest for the batch's class: the first
    plan of a new class measures, the next one reads the same choice from the table (and the
    table file holds it); results match the oracle on the same sketches with the chosen
    configuration."""
    import os
    g = np.random.default_rng(7)
    mats, ks = [], []
    for i in range(40):
        m = int(g.integers(900, 1000))
        n = int(g.integers(450, 500))
        A = spectrum_matrix(m, n, 0.9 ** np.arange(min(m, n)), seed=2000 + i)
        mats.append(A.astype(np.float32).astype(np.float64))
        ks.append(42 if i == 0 else int(g.integers(20, 42)))     # k + p = 50 at most
    p, q, seed = 8, 1, 0x55AA
    info = []
    Us, Ss, Vs = run_batch(engine, mats, ks, p, q, seed, info)
    run_batch(engine, mats, ks, p, q, seed + 1, info)            # the same class
    (lp1, cu1, t1, ms1), (lp2, cu2, t2, ms2) = info
    assert lp1 in (4, 8, 16, 32) and cu1 in (0, 1) and t1 == 1 and ms1 > 0
    assert (lp2, cu2, t2) == (lp1, cu1, 2)
    with open(os.environ["RSVDPACK_TUNE_FILE"]) as f:
        assert any(line.split()[1:3] == [str(lp1), str(cu1)] for line in f if line.startswith("l50_"))
    for i in (0, 17, 39):
        A, k = mats[i], ks[i]
        n = A.shape[1]
        port.set_omega(ListOmega([philox_gaussians(n * (k + p), seed, i)]))
        Uo, So, Vo = port.low_rank_svd_rand_decomp_fixed_rank(A, k, p, 1, q, 1)
        so = np.diag(So)
        assert np.max(np.abs(Ss[i] - so) / so[0]) < 2e-4
