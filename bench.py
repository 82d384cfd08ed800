#!/usr/bin/env python
"""Benchmark: rSVD solves/sec on the mixed-precision single large rSVD workload.

Workload (one "step" = one fixed-rank randomized SVD with the reference's semantics):
  A 16384 x 8192 FP32 = U diag(s) V^T + 1e-4 G, s_i = i^-1.5, Haar U, V, G standard
  Gaussian (seeded synthetic data); k=256, p=16, q=2 (reference semantics: one power
  round), s=1, vnum=1.
  value : solves/s with A resident in HBM, through rsvdpack_dev_svd_fixed_rank.
  e2e   : solves/s through the reference C API (low_rank_svd_rand_decomp_fixed_rank)
          from a pinned host FP64 matrix: H2D of A, solve, D2H of U, S, V every step.
  A (512 MiB) is larger than L2 (129 MB), so no flush is needed between steps.
  Residual ||A - U S V^T||_F / ||A||_F and the top-k singular values (against FP64 LAPACK) are
  checked against the FP64 path of the same method on the same test matrix ("matched
  FP64-oracle error").

--impl reference times the CPU oracle (oracle/port: the reference's algorithm on
OpenBLAS, all host cores) on the same workload and prints the same JSON line.
Multi-GPU (torchrun): independent replicas, one matrix per rank ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

M_ROWS, N_COLS, K, P, Q, S_ORTH, VNUM = 16384, 8192, 256, 16, 2, 1, 1
METRIC = "rSVD solves/sec at matched FP64-oracle error (16384x8192 FP32, k=256, p=16, q=2)"
# DRAM bytes (read + write) per tensor-core sketch launch on this workload, mean of the A*X
# (BF16 A: 276.3 MB) and A^T*X (TF32: 605.9 MB) forms, from one ncu capture of this script
# (profiles/tc_gemm_sketch_16384x8192.txt).
TC_TRAFFIC_PER_LAUNCH = 441.1e6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default=os.environ.get("RSVDPACK_BENCH_PRECISION", "tf32"),
                    choices=["fp64", "fp32", "tf32", "bf16"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-c1", action="store_true", help="skip the 2000 x 1000 FP64 fixed-rank leg")
    ap.add_argument("--no-c5", action="store_true", help="skip the 20000 x 10000 two-sided ID / CUR leg")
    # bracket one leg's timed region with cudaProfilerStart/Stop (ncu --profile-from-start off)
    ap.add_argument("--profile-leg", choices=["solve", "learned", "batched"], default=None)
    # run one fixed profiling case (see PROFILE_CASES) and exit
    ap.add_argument("--profile-case", choices=["update", "gemm3x", "solve", "pivot", "norm", "df64", "lxl"],
                    default=None)
    return ap.parse_args()


def job_throughput(ms_local, world, torch, device):
    """Whole-job solves/s from this rank's ms per solve: the slowest rank's time (MAX over
    ranks; every rank runs the same per-rank work, so the job rate is world / slowest)."""
    ms = float(ms_local)
    if world > 1:
        t = torch.tensor([ms], device=device, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * 1000.0 / ms


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def make_matrix(torch, device, seed):
    """A = U diag(i^-1.5) V^T + 1e-4 G in FP32 on the GPU (Haar U, V from QR of Gaussians)."""
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    m, n = M_ROWS, N_COLS
    Ug, _ = torch.linalg.qr(torch.randn(m, n, device=device, generator=g))
    Vg, _ = torch.linalg.qr(torch.randn(n, n, device=device, generator=g))
    s = torch.arange(1, n + 1, device=device, dtype=torch.float32) ** -1.5
    A = (Ug * s) @ Vg.T + 1e-4 * torch.randn(m, n, device=device, generator=g)
    del Ug, Vg
    # column-major storage: the transpose of a row-major n x m tensor
    At = A.T.contiguous()          # At[j, i] = A[i, j]; memory = A column-major, ld = m
    del A
    torch.cuda.synchronize()
    return At


class ClockSampler:
    """nvidia-smi sampling during the timed region (SM clock, throttle reasons)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


def solve_roofline(m, n, k, l, q, s, vnum, esize, ms, hbm_gbs, tensor_tflops):
    """Whole-solve roofline of one fixed-rank rSVD (the reference's semantics: q - 1 power
    rounds, an orthonormalisation where (2j-2) % s == 0 / (2j-1) % s == 0).  Algorithmic work:
      products: 2q passes over A (Y = A Omega, 2(q-1) power products, B^T = A^T Q), each
                2 m n l flops and m n esize bytes;
      QR:       4 r l^2 flops per orthonormalisation of an r x l basis (the Householder count;
                the engine's CholeskyQR2 is charged the same);
      l x l:    22 l^3 (nominal SVD count) and the factor products 2 (m + n) l k.
    roofline time = max(flops / tensor peak, bytes / HBM peak); frac = roofline / measured."""
    orth_rows = []
    for j in range(1, q):
        if (2 * j - 2) % s == 0:
            orth_rows.append(m)
        if (2 * j - 1) % s == 0:
            orth_rows.append(n)
    orth_rows.append(m)
    if vnum == 1 or vnum > 2:
        orth_rows.append(n)
    passes = 2 * q
    flops = (passes * 2.0 * m * n * l + sum(4.0 * r * l * l for r in orth_rows)
             + 22.0 * l ** 3 + 2.0 * (m + n) * l * k)
    nbytes = passes * float(m) * n * esize
    t_flops = flops / (tensor_tflops * 1e12) * 1e3
    t_bytes = nbytes / (hbm_gbs * 1e9) * 1e3
    t_roof = max(t_flops, t_bytes)
    return {"flops": flops, "bytes": nbytes, "passes": passes, "roofline_ms": t_roof,
            "bound": "tensor" if t_flops >= t_bytes else "hbm", "measured_ms": ms, "frac": t_roof / ms,
            "tensor_peak_tflops": tensor_tflops, "hbm_peak_gbs": hbm_gbs}


def cpu_solve_seconds(A_host, threads, repeats=1):
    """Time the CPU oracle (oracle/port) on the workload; returns seconds per solve."""
    from lowrankmatrixdecompositioncodes_gb300.capi import RsvdLibrary, SeededOmega
    so = os.path.join(ROOT, "oracle", "port", "librsvd_port.so")
    if not os.path.exists(so):
        subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"])
    port = RsvdLibrary(so)
    port.lib.rsvdpack_set_num_threads(threads)
    port.set_omega(SeededOmega(1234))
    M = port.to_mat(A_host)
    from lowrankmatrixdecompositioncodes_gb300.capi import PMat
    times = []
    for _ in range(repeats):
        U, S, V, fr = PMat(), PMat(), PMat(), C.c_int(0)
        t0 = time.perf_counter()
        port.lib.low_rank_svd_rand_decomp_fixed_rank(M, K, P, VNUM, Q, S_ORTH, C.byref(fr), C.byref(U),
                                                     C.byref(S), C.byref(V))
        times.append(time.perf_counter() - t0)
        for x in (U, S, V):
            port.lib.matrix_delete(x)
    port.lib.matrix_delete(M)
    return times


WEIGHTS = os.path.join(ROOT, "lowrankmatrixdecompositioncodes_gb300", "learned", "proposal_mlp.bin")


def learned_qb_leg(torch, eng, dev, steps=2, profile=False):
    """Fixed-precision blocked QB on the 32768 x 16384 FP32 workload (s_i = exp(-i/200), Haar
    factors): the plain FP32 adaptive loop (randQB_pb_new semantics, kstep = 128, q = 1) against the
    learned proposal in TF32 mode at TOL = 1e-5 ||A||_F, then the plain loop on the same values as
    FP64 data in the FP64 and FP64X modes at TOL = 1e-6 ||A||_F (FP32-arithmetic deflation
    updates A_res -= Q_j B_j err by ~u sqrt(w/2) of their size, and the first blocks remove ~0.5
    ||A||: a floor near 1e-6 ||A||_F at this size).  Every residual is checked in FP64; times are
    per solve with A resident (CUDA events).  The matrix is formed in FP64 at rank 4000
    (s_4000 = 2e-9) and rounded once to FP32 (rounding noise ~4e-8 ||A||_F); an FP32 product of
    the factors would add a full-rank accumulation noise of ~5e-6 ||A||_F."""
    L = eng.lib
    m, n, r = 32768, 16384, 4000
    g = torch.Generator(device=dev)
    g.manual_seed(3)
    U, _ = torch.linalg.qr(torch.randn(m, r, device=dev, generator=g, dtype=torch.float64))
    V, _ = torch.linalg.qr(torch.randn(n, r, device=dev, generator=g, dtype=torch.float64))
    sv = torch.exp(-torch.arange(r, device=dev, dtype=torch.float64) / 200.0)
    At = ((U * sv) @ V.T).T.float().contiguous()
    del U, V
    torch.cuda.empty_cache()
    fro = float(torch.linalg.norm(At.double()))
    tol_rel = 1e-5
    L.rsvdpack_dev_qb.argtypes = [C.c_void_p, C.c_int, C.c_longlong, C.c_int, C.c_int, C.c_int, C.c_int,
                                  C.c_double, C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong,
                                  C.c_int, C.POINTER(C.c_int)]
    cap = 6144
    Q = torch.empty(cap, m, device=dev)
    B = torch.empty(n, cap, device=dev)
    stream = torch.cuda.ExternalStream(L.rsvdpack_stream())
    out = {"workload": "fixed-precision QB 32768x16384 FP32, s_i = exp(-i/200), TOL = 1e-5 ||A||_F",
           "matrix": "formed in FP64 (rank 4000), rounded once to FP32"}
    for name, learned, prec in (("plain_fp32", False, "fp32"), ("learned_tf32", True, "tf32")):
        eng.set_precision(prec)
        eng.set_learned(learned)
        fr = C.c_int(0)
        times = []
        for i in range(steps + 1):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            prof = profile and learned and i == steps
            if prof:
                torch.cuda.cudart().cudaProfilerStart()
            e0.record(stream)
            rc = L.rsvdpack_dev_qb(At.data_ptr(), 1, m, m, n, 128, 0, tol_rel * fro, 1, 1, Q.data_ptr(), m,
                                   B.data_ptr(), cap, cap, C.byref(fr))
            e1.record(stream)
            e1.synchronize()
            if prof:
                torch.cuda.cudart().cudaProfilerStop()
            if rc:
                raise RuntimeError(f"QB failed: {eng.last_error()}")
            if i > 0:
                times.append(e0.elapsed_time(e1))
        path = eng.last_timing().learned_path
        k = fr.value
        Qm, Bm = Q[:k].T, B[:, :k].T
        res = 0.0
        for c0 in range(0, n, 2048):
            c1 = min(n, c0 + 2048)
            E = At[c0:c1].T.double() - Qm.double() @ Bm[:, c0:c1].double()
            res += float((E * E).sum())
        out[name] = {"ms_per_solve": sum(times) / len(times), "rank": k, "rel_residual": res ** 0.5 / fro,
                     "meets_tol": bool(res ** 0.5 <= tol_rel * fro), "learned_path": path}
    eng.set_learned(False)
    eng.set_precision("fp64")
    out["speedup"] = out["plain_fp32"]["ms_per_solve"] / out["learned_tf32"]["ms_per_solve"]
    del Q, B
    torch.cuda.empty_cache()
    # TOL = 1e-6 on FP64 data: the reference's loop (kstep 128, q = 1) with FP64 products against
    # the FP64X mode's double-float products, one solve each, residual checked in FP64
    try:
        out["fp64_tol1e-6"] = fp64_tol_leg(torch, eng, L, At, m, n, fro, stream, dev)
    except Exception as e:
        out["fp64_tol1e-6"] = {"error": f"{type(e).__name__}: {e}"}
    eng.set_precision("fp64")
    torch.cuda.empty_cache()
    return out


def fp64_tol_leg(torch, eng, L, At, m, n, fro, stream, dev):
    """TOL = 1e-6 on FP64 data: the reference's loop (kstep 128, q = 1) with FP64 products against
    the FP64X mode's double-float products, one solve each, residual checked in FP64."""
    tol6 = 1e-6
    A64 = At.double()
    del At
    torch.cuda.empty_cache()
    cap64 = 6144
    Q64 = torch.empty(cap64, m, device=dev, dtype=torch.float64)
    B64 = torch.empty(n, cap64, device=dev, dtype=torch.float64)
    leg6 = {"workload": "the same FP32 values as FP64 data, TOL = 1e-6 ||A||_F, plain blocked QB, kstep 128, q = 1"}
    for name, prec in (("fp64x", "fp64x"), ("fp64", "fp64")):
        eng.set_precision(prec)
        fr = C.c_int(0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        rc = L.rsvdpack_dev_qb(A64.data_ptr(), 0, m, m, n, 128, 0, tol6 * fro, 1, 1, Q64.data_ptr(), m,
                               B64.data_ptr(), cap64, cap64, C.byref(fr))
        e1.record(stream)
        e1.synchronize()
        if rc:
            raise RuntimeError(f"FP64 QB failed: {eng.last_error()}")
        k = fr.value
        Qm, Bm = Q64[:k].T, B64[:, :k].T
        res = 0.0
        for c0 in range(0, n, 2048):
            c1 = min(n, c0 + 2048)
            E = A64[c0:c1].T - Qm @ Bm[:, c0:c1]
            res += float((E * E).sum())
        leg6[name] = {"ms_per_solve": e0.elapsed_time(e1), "rank": k, "rel_residual": res ** 0.5 / fro,
                      "meets_tol": bool(res ** 0.5 <= tol6 * fro)}
    leg6["speedup_fp64x_vs_fp64"] = leg6["fp64"]["ms_per_solve"] / leg6["fp64x"]["ms_per_solve"]
    del A64, Q64, B64
    return leg6


def batched_leg(torch, eng, dev, execs=5, profile=False):
    """Batched rSVD workload: 4096 FP32 matrices, m ~ U[64, 1024], n ~ U[32, 512] (seed 0),
    s_i = 0.9^i with Haar factors, k = floor(min(m, n) / 8), p = 8, q = 1; one graph-captured
    persistent launch per execute.  Residuals of four items are checked against the optimal
    rank-k tail of their spectrum."""
    import numpy as np
    L = eng.lib
    L.rsvdpack_batch_plan_create.restype = C.c_void_p
    L.rsvdpack_batch_plan_create.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_ulonglong]
    L.rsvdpack_batch_plan_execute.restype = C.c_int
    L.rsvdpack_batch_plan_execute.argtypes = [C.c_void_p]
    L.rsvdpack_batch_plan_destroy.argtypes = [C.c_void_p]
    cnt = 4096
    g = np.random.default_rng(0)
    ms, ns = g.integers(64, 1025, cnt), g.integers(32, 513, cnt)
    ks = [max(1, int(min(a, b)) // 8) for a, b in zip(ms, ns)]
    gen = torch.Generator(device=dev)
    gen.manual_seed(0)
    dA, dU, dV, dS = [], [], [], []
    for m, n, k in zip(ms, ns, ks):
        r = int(min(m, n))
        Uq, _ = torch.linalg.qr(torch.randn(int(m), r, device=dev, generator=gen))
        Vq, _ = torch.linalg.qr(torch.randn(int(n), r, device=dev, generator=gen))
        sv = 0.9 ** torch.arange(r, device=dev, dtype=torch.float32)
        dA.append(((Uq * sv) @ Vq.T).T.contiguous())
        dU.append(torch.zeros(k, int(m), device=dev))
        dV.append(torch.zeros(k, int(n), device=dev))
        dS.append(torch.zeros(k, device=dev, dtype=torch.float64))
    arr = lambda vals, t: (t * cnt)(*vals)
    ptr = lambda ts: (C.c_void_p * cnt)(*[t.data_ptr() for t in ts])
    mi = arr([int(x) for x in ms], C.c_int)
    ni = arr([int(x) for x in ns], C.c_int)
    torch.cuda.synchronize()
    plan = L.rsvdpack_batch_plan_create(cnt, mi, ni, arr(ks, C.c_int), 8, 1, 1, ptr(dA),
                                        arr([int(x) for x in ms], C.c_longlong), ptr(dU),
                                        arr([int(x) for x in ms], C.c_longlong), ptr(dS), ptr(dV),
                                        arr([int(x) for x in ns], C.c_longlong), 7)
    if not plan:
        raise RuntimeError(f"batch plan failed: {eng.last_error()}")
    L.rsvdpack_batch_plan_info.restype = C.c_int
    L.rsvdpack_batch_plan_info.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                           C.POINTER(C.c_double)]
    lp, cu, tuned, tms = C.c_int(0), C.c_int(0), C.c_int(0), C.c_double(0)
    L.rsvdpack_batch_plan_info(plan, C.byref(lp), C.byref(cu), C.byref(tuned), C.byref(tms))
    tuner = {"lanes_per_jacobi_pair": lp.value, "column_group_offset": cu.value,
             "source": {0: "default", 1: "measured at plan creation", 2: "tuning table"}[tuned.value],
             "sample_ms": tms.value}
    stream = torch.cuda.ExternalStream(L.rsvdpack_stream())
    try:
        for _ in range(3):
            if L.rsvdpack_batch_plan_execute(plan):
                raise RuntimeError(eng.last_error())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(execs):
            if L.rsvdpack_batch_plan_execute(plan):
                raise RuntimeError(eng.last_error())
        e1.record(stream)
        e1.synchronize()
        ms_exec = e0.elapsed_time(e1) / execs
        if profile:
            torch.cuda.synchronize()
            torch.cuda.cudart().cudaProfilerStart()
            if L.rsvdpack_batch_plan_execute(plan):
                raise RuntimeError(eng.last_error())
            torch.cuda.synchronize()
            torch.cuda.cudart().cudaProfilerStop()
    finally:
        L.rsvdpack_batch_plan_destroy(plan)
    checks = []
    for i in (0, 1, cnt // 2, cnt - 1):
        A = dA[i].T.double()
        res = float(torch.linalg.norm(A - (dU[i].T.double() * dS[i]) @ dV[i].double()) / torch.linalg.norm(A))
        r = int(min(ms[i], ns[i]))
        sv = 0.9 ** np.arange(r)
        checks.append({"item": i, "rel_residual": res, "optimal": float(np.sqrt(np.sum(sv[ks[i]:] ** 2) / np.sum(sv ** 2)))})
    nbytes = sum(int(a) * int(b) for a, b in zip(ms, ns)) * 4
    return {"workload": "4096 matrices m~U[64,1024] n~U[32,512], s_i = 0.9^i, k = min(m,n)/8, p = 8, q = 1",
            "ms_per_batch": ms_exec, "solves_per_s": cnt * 1000.0 / ms_exec, "bytes_of_A": nbytes,
            "autotuner": tuner,
            "residual_checks": checks}


# ------------------------------------------------------------------ checkers and extra legs
def port_library():
    """The CPU oracle (oracle/port: the reference's algorithms restated in C on OpenBLAS)."""
    from lowrankmatrixdecompositioncodes_gb300.capi import RsvdLibrary
    so = os.path.join(ROOT, "oracle", "port", "librsvd_port.so")
    if not os.path.exists(so):
        subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"])
    return RsvdLibrary(so)


def top_singular_values_fp64(torch, At, k):
    """Checker: the top k singular values of A (At = column-major A as an n x m row-major tensor)
    in FP64 -- A^T A formed in FP64 on the GPU, its top k eigenvalues by LAPACK dsyevr on the host
    (scipy), square-rooted.  Relative accuracy ~eps (s_1 / s_i)^2: ~1e-12 for the workloads here."""
    import numpy as np
    import scipy.linalg as sla
    Ad = At.double()
    G = (Ad @ Ad.T).cpu().numpy()
    del Ad
    n = G.shape[0]
    ev = sla.eigh(G, eigvals_only=True, subset_by_index=[n - k, n - 1], driver="evr", overwrite_a=True)
    return np.sqrt(np.maximum(ev[::-1], 0.0))


def sigma_rel_err(got, want):
    import numpy as np
    got = np.sort(np.asarray(got, dtype=float))[::-1][:len(want)]
    return float(np.max(np.abs(got - want) / want))


def sigma_rel_err_mean(got, want):
    import numpy as np
    got = np.sort(np.asarray(got, dtype=float))[::-1][:len(want)]
    return float(np.mean(np.abs(got - want) / want))


def dev_residual_norms(eng, A_ptr, dt, lda, m, n, U_ptr, ldu, S_ptr, V_ptr, ldv, k, iters=20):
    L = eng.lib
    L.rsvdpack_dev_residual_norms.restype = C.c_int
    L.rsvdpack_dev_residual_norms.argtypes = [C.c_void_p, C.c_int, C.c_longlong, C.c_int, C.c_int, C.c_void_p,
                                              C.c_longlong, C.c_void_p, C.c_void_p, C.c_longlong, C.c_int, C.c_int,
                                              C.POINTER(C.c_double), C.POINTER(C.c_double)]
    fro, spec = C.c_double(0), C.c_double(0)
    rc = L.rsvdpack_dev_residual_norms(A_ptr, dt, lda, m, n, U_ptr, ldu, S_ptr, V_ptr, ldv, k, iters, C.byref(fro),
                                       C.byref(spec))
    if rc:
        raise RuntimeError(f"residual norms failed: {eng.last_error()}")
    return fro.value, spec.value


def host_residuals(torch, eng, A, U, S, V, fro_a, spec_a):
    """Relative Frobenius and spectral residual of a host factorisation A ~ U diag(S) V^T through
    the engine's residual reporter (FP64 device data)."""
    import numpy as np
    dev = "cuda"
    col = lambda X: torch.from_numpy(np.ascontiguousarray(X.T)).to(dev)
    m, n = A.shape
    k = U.shape[1]
    dA, dU, dV = col(A), col(U), col(V)
    dS = torch.from_numpy(np.asarray(S, dtype=np.float64).copy()).to(dev)
    fro, spec = dev_residual_norms(eng, dA.data_ptr(), 0, m, m, n, dU.data_ptr(), m, dS.data_ptr(), dV.data_ptr(), n, k)
    del dA, dU, dV, dS
    return fro / fro_a, spec / spec_a


def timed_c_call(fn, *args, reps=1):
    """Seconds per call of a reference-API routine (host mat in, host mats out), outputs freed."""
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn(*args)
        ts.append(time.perf_counter() - t0)
    return ts


def plain_fixed_rank_leg(torch, eng, reps=10):
    """Plain fixed-rank rSVD at the reference's own CPU-runnable size: A 2000 x 1000 FP64 =
    U diag(10^(-6(i-1)/999)) V^T (Haar U, V from QR of seeded Gaussians), k=100, p=10, q=2, s=1,
    vnum=1.  FP64 mode (the reference's arithmetic) and FP64X mode (double-float products, refined
    l x l SVD): parity against the oracle on the same supplied test matrix, top-100 singular values
    and residuals against FP64 LAPACK, and the C-API call timed from a host matrix, next to the
    oracle on all host cores and on one."""
    import numpy as np
    from lowrankmatrixdecompositioncodes_gb300.capi import PMat, SeededOmega
    m, n, k, p, q = 2000, 1000, 100, 10, 2
    g = np.random.default_rng(2024)
    s_all = 10.0 ** (-6.0 * np.arange(n) / (n - 1))
    U0, _ = np.linalg.qr(g.standard_normal((m, n)))
    V0, _ = np.linalg.qr(g.standard_normal((n, n)))
    A = (U0 * s_all) @ V0.T
    sv = np.linalg.svd(A, compute_uv=False)                  # FP64 LAPACK
    fro_a, spec_a = float(np.linalg.norm(A)), float(sv[0])
    opt_fro = float(np.sqrt(np.sum(sv[k:] ** 2)) / fro_a)
    port = port_library()
    threads = os.cpu_count() or 1
    port.lib.rsvdpack_set_num_threads(threads)
    port.set_omega(SeededOmega(99))
    Uo, So, Vo = port.low_rank_svd_rand_decomp_fixed_rank(A, k, p, 1, q, 1)
    so = np.diag(So)
    out = {"workload": "plain fixed-rank rSVD 2000x1000 FP64, s_i = 10^(-6(i-1)/999), k=100 p=10 q=2 s=1 vnum=1",
           "lapack_optimal_rel_frobenius": opt_fro,
           "oracle": {"sigma_rel_err_top100": sigma_rel_err(so, sv[:k])}}
    out["oracle"]["rel_frobenius"], out["oracle"]["rel_spectral"] = host_residuals(torch, eng, A, Uo, so, Vo, fro_a,
                                                                                   spec_a)

    def c_call(lib, M):
        U, S, V, fr = lib.PMat(), lib.PMat(), lib.PMat(), lib.Int(0)
        lib.lib.low_rank_svd_rand_decomp_fixed_rank(M, k, p, 1, q, 1, C.byref(fr), C.byref(U), C.byref(S),
                                                    C.byref(V))
        for x in (U, S, V):
            lib.lib.matrix_delete(x)

    for prec in ("fp64", "fp64x"):
        eng.set_precision(prec)
        eng.set_use_provider(True)
        eng.set_omega(SeededOmega(99))
        Ue, Se, Ve = eng.low_rank_svd_rand_decomp_fixed_rank(A, k, p, 1, q, 1)
        eng.check()
        se = np.diag(Se)
        leg = {"parity_sigma_vs_oracle": float(np.max(np.abs(se - so) / so)),
               "sigma_rel_err_top100": sigma_rel_err(se, sv[:k])}
        leg["rel_frobenius"], leg["rel_spectral"] = host_residuals(torch, eng, A, Ue, se, Ve, fro_a, spec_a)
        leg["parity_ok"] = leg["parity_sigma_vs_oracle"] < 1e-10
        eng.set_use_provider(False)
        M = eng.to_mat(A)
        c_call(eng, M)
        ts = timed_c_call(c_call, eng, M, reps=reps)
        eng.lib.matrix_delete(M)
        eng.check()
        leg["c_api_ms"] = 1e3 * float(np.median(ts))
        leg["solves_per_s"] = 1.0 / float(np.median(ts))
        leg["h2d_bytes_per_call"] = m * n * 8
        out[prec] = leg
    eng.set_precision("fp64")
    eng.set_use_provider(False)
    port.set_omega(None)
    M = port.to_mat(A)
    for cores in (threads, 1):
        port.lib.rsvdpack_set_num_threads(cores)
        c_call(port, M)
        ts = timed_c_call(c_call, port, M, reps=5)
        out["cpu_cores_%d" % cores] = {"ms": 1e3 * float(np.median(ts)), "solves_per_s": 1.0 / float(np.median(ts)),
                                       "cores": cores, "kind": "port"}
    port.lib.matrix_delete(M)
    port.lib.rsvdpack_set_num_threads(threads)
    out["speedup_fp64x_vs_cpu_all_cores"] = out["fp64x"]["solves_per_s"] / out["cpu_cores_%d" % threads]["solves_per_s"]
    return out


def id_cur_leg(torch, eng):
    """Two-sided ID and CUR: A 20000 x 10000 = U diag(i^-2) V^T (Haar factors; the spectrum
    truncated at rank 1000, where i^-2 is 1e-6, so the singular values are known exactly), k=500,
    p=20, q=2, s=1.  The engine (FP64X mode: the sketch passes as double-float products; and the
    FP64 mode) and the oracle on all host cores get the same supplied test matrices: index sets
    must be identical; times are of the C-API call from a host matrix; the CUR residual is
    measured by the engine's residual reporter and set against the rank-500 optimum."""
    import numpy as np
    from lowrankmatrixdecompositioncodes_gb300.capi import SeededOmega
    m, n, k, p, q, r = 20000, 10000, 500, 20, 2, 1000
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    Uq, _ = torch.linalg.qr(torch.randn(m, r, device="cuda", dtype=torch.float64, generator=g))
    Vq, _ = torch.linalg.qr(torch.randn(n, r, device="cuda", dtype=torch.float64, generator=g))
    s = torch.arange(1, r + 1, device="cuda", dtype=torch.float64) ** -2.0
    A = ((Uq * s) @ Vq.T).cpu().numpy()
    del Uq, Vq
    torch.cuda.empty_cache()
    sv = s.cpu().numpy()
    fro_a, spec_a = float(np.sqrt(np.sum(sv ** 2))), float(sv[0])
    out = {"workload": "two-sided ID and CUR 20000x10000, s_i = i^-2 (rank 1000), k=500 p=20 q=2 s=1",
           "rank_k_optimal_rel_frobenius": float(np.sqrt(np.sum(sv[k:] ** 2)) / fro_a),
           "rank_k_optimal_rel_spectral": float(sv[k] / spec_a)}
    port = port_library()
    threads = os.cpu_count() or 1
    port.lib.rsvdpack_set_num_threads(threads)

    def run(lib, name, seed):
        lib.set_omega(SeededOmega(seed))
        M = lib.to_mat(A)
        if name == "id":
            o = [lib.PVec(), lib.PVec(), lib.PMat(), lib.PMat()]
            fn = lambda: lib.lib.id_two_sided_rand_decomp_fixed_rank(M, k, p, q, 1, *[C.byref(x) for x in o])
        else:
            o = [lib.PMat(), lib.PMat(), lib.PMat()]
            fn = lambda: lib.lib.cur_rand_decomp_fixed_rank(M, k, p, q, 1, *[C.byref(x) for x in o])
        t0 = time.perf_counter()
        fn()
        t = time.perf_counter() - t0
        lib.lib.matrix_delete(M)
        if name == "id":
            res = (lib.from_vec(o[0]), lib.from_vec(o[1]), lib.from_mat(o[2]), lib.from_mat(o[3]))
        else:
            res = tuple(lib.from_mat(x) for x in o)
        return t, res

    t_id_o, id_o = run(port, "id", 2026)
    t_cur_o, cur_o = run(port, "cur", 2027)
    out["cpu_all_cores"] = {"cores": threads, "kind": "port", "id_ms": 1e3 * t_id_o, "cur_ms": 1e3 * t_cur_o}

    def cur_res(Cm, Um, Rm):
        # A ~ C U R = (C) diag(1) (R^T U^T)^T
        return host_residuals(torch, eng, A, Cm, np.ones(Cm.shape[1]), (Um @ Rm).T, fro_a, spec_a)

    out["oracle_cur_rel_frobenius"], out["oracle_cur_rel_spectral"] = cur_res(*cur_o)
    for prec in ("fp64x", "fp64"):
        eng.set_precision(prec)
        eng.set_use_provider(True)
        run(eng, "id", 2026)                     # warm-up (module loads, pools)
        t_id, id_e = run(eng, "id", 2026)
        t_cur, cur_e = run(eng, "cur", 2027)
        eng.check()
        leg = {"id_ms": 1e3 * t_id, "cur_ms": 1e3 * t_cur,
               "index_sets_identical": bool(np.array_equal(id_e[0], id_o[0]) and np.array_equal(id_e[1], id_o[1])),
               "cur_gathers_identical": bool(np.array_equal(cur_e[0], cur_o[0]) and np.array_equal(cur_e[2], cur_o[2])),
               "h2d_bytes_per_call": m * n * 8}
        leg["cur_rel_frobenius"], leg["cur_rel_spectral"] = cur_res(*cur_e)
        leg["speedup_id_vs_cpu"] = t_id_o / t_id
        leg["speedup_cur_vs_cpu"] = t_cur_o / t_cur
        out[prec] = leg
    eng.set_precision("fp64")
    eng.set_use_provider(False)
    port.set_omega(None)
    del A
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import numpy as np
    import torch
    dev = "cuda:0" if torch.cuda.is_available() else "cpu"
    if dev.startswith("cuda"):
        At = make_matrix(torch, dev, seed=1)
        A_host = At.T.double().cpu().numpy()       # m x n view of column-major data
        del At
        torch.cuda.empty_cache()
    else:
        g = np.random.default_rng(1)
        A_host = g.standard_normal((M_ROWS, N_COLS))
    threads = os.cpu_count() or 1
    t_all = cpu_solve_seconds(A_host, threads, repeats=args.warmup + args.steps)
    t = t_all[args.warmup:]
    sec = sum(t) / len(t)
    val = 1.0 / sec
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * sec, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "single large rSVD 16384x8192 k=256 p=16 q=2 s=1 vnum=1", "m": M_ROWS,
                   "n": N_COLS, "k": K, "p": P, "q": Q, "s": S_ORTH},
        "cpu_baseline": {"value": val, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full solves of the workload (after {args.warmup} warm-up)"},
        "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    rank, world, local = dist_env()
    os.environ["RSVDPACK_DEVICE"] = str(local)
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device(dev))
    from lowrankmatrixdecompositioncodes_gb300 import load_engine
    from lowrankmatrixdecompositioncodes_gb300.capi import PMat

    eng = load_engine()
    sms, name, cc = eng.device_info()
    if sms <= 0:
        raise RuntimeError(f"engine unavailable: {eng.last_error()}")
    eng.set_precision(args.precision)
    eng.set_use_provider(False)
    L = eng.lib
    L.rsvdpack_dev_svd_fixed_rank.restype = C.c_int
    L.rsvdpack_dev_svd_fixed_rank.argtypes = [C.c_void_p, C.c_int, C.c_longlong, C.c_int, C.c_int, C.c_int, C.c_int,
                                              C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p,
                                              C.c_void_p, C.c_longlong]
    L.rsvdpack_dev_sketch.restype = C.c_int
    L.rsvdpack_dev_sketch.argtypes = [C.c_void_p, C.c_int, C.c_longlong, C.c_int, C.c_int, C.c_void_p,
                                      C.c_longlong, C.c_int, C.c_void_p, C.c_longlong, C.c_int]
    L.rsvdpack_stream.restype = C.c_void_p
    L.rsvdpack_reset_omega_counter.restype = None

    m, n, k, l = M_ROWS, N_COLS, K, K + P
    At = make_matrix(torch, dev, seed=1 + rank)        # column-major A, ld = m
    dA = At.data_ptr()
    dt = 0 if args.precision == "fp64" else 1
    if dt == 0:
        At64 = At.double()
        dA = At64.data_ptr()
    tdt = torch.float64 if dt == 0 else torch.float32
    U = torch.empty(k, m, device=dev, dtype=tdt)        # column-major m x k
    V = torch.empty(k, n, device=dev, dtype=tdt)
    Sv = torch.empty(k, device=dev, dtype=torch.float64)
    stream = torch.cuda.ExternalStream(L.rsvdpack_stream())

    def solve():
        rc = L.rsvdpack_dev_svd_fixed_rank(dA, dt, m, m, n, k, P, VNUM, Q, S_ORTH, U.data_ptr(), m,
                                           Sv.data_ptr(), V.data_ptr(), n)
        if rc:
            raise RuntimeError(f"solve failed: {eng.last_error()}")

    def residual():
        Ur, Vr = U.T.double(), V.T.double()
        Ad = At.T.double()
        R = Ad - (Ur * Sv) @ Vr.T
        return float(torch.linalg.norm(R) / torch.linalg.norm(Ad))

    # matched-error check: same test matrix for the working precision and for FP64; singular
    # values against FP64 LAPACK (top k of A^T A by dsyevr), residuals by the engine's reporter
    sv_lapack = top_singular_values_fp64(torch, At, k) if rank == 0 else None
    fro_a = float(torch.linalg.norm(At.double()))
    L.rsvdpack_reset_omega_counter()
    solve()
    res_mixed = residual()
    fro_m, spec_m = dev_residual_norms(eng, dA, dt, m, m, n, U.data_ptr(), m, Sv.data_ptr(), V.data_ptr(), n, k)
    sig_mixed = sigma_rel_err(Sv.cpu().numpy(), sv_lapack) if sv_lapack is not None else None
    sig_mixed16 = sigma_rel_err(Sv.cpu().numpy()[:16], sv_lapack[:16]) if sv_lapack is not None else None
    sig_mixed_mean = sigma_rel_err_mean(Sv.cpu().numpy(), sv_lapack) if sv_lapack is not None else None
    res_fp64 = spec_fp64 = sig_fp64 = sig_fp64_16 = sig_fp64_mean = None
    if args.precision != "fp64":
        eng.set_precision("fp64")
        A64 = At.double()
        U64 = torch.empty(k, m, device=dev, dtype=torch.float64)
        V64 = torch.empty(k, n, device=dev, dtype=torch.float64)
        S64 = torch.empty(k, device=dev, dtype=torch.float64)
        L.rsvdpack_reset_omega_counter()
        rc = L.rsvdpack_dev_svd_fixed_rank(A64.data_ptr(), 0, m, m, n, k, P, VNUM, Q, S_ORTH, U64.data_ptr(), m,
                                           S64.data_ptr(), V64.data_ptr(), n)
        if rc:
            raise RuntimeError(f"fp64 solve failed: {eng.last_error()}")
        R = A64.T - (U64.T * S64) @ V64
        res_fp64 = float(torch.linalg.norm(R) / torch.linalg.norm(A64))
        del R
        _, spec_fp64 = dev_residual_norms(eng, A64.data_ptr(), 0, m, m, n, U64.data_ptr(), m, S64.data_ptr(),
                                          V64.data_ptr(), n, k)
        if sv_lapack is not None:
            sig_fp64 = sigma_rel_err(S64.cpu().numpy(), sv_lapack)
            sig_fp64_16 = sigma_rel_err(S64.cpu().numpy()[:16], sv_lapack[:16])
            sig_fp64_mean = sigma_rel_err_mean(S64.cpu().numpy(), sv_lapack)
        del A64, U64, V64, S64
        eng.set_precision(args.precision)
        torch.cuda.empty_cache()

    # ---------------- device-resident timed region
    for _ in range(args.warmup):
        solve()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.4)
    launches = 0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    if args.profile_leg == "solve":
        torch.cuda.cudart().cudaProfilerStart()
    ev0.record(stream)
    phase_sum = {"products": 0.0, "orthonormalisation": 0.0, "lxl_svd": 0.0}
    for _ in range(args.steps):
        solve()
        tm = eng.last_timing()
        launches += tm.kernel_launches
        phase_sum["products"] += tm.sketch_ms
        phase_sum["orthonormalisation"] += tm.orth_ms
        phase_sum["lxl_svd"] += tm.small_ms
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    if args.profile_leg == "solve":
        torch.cuda.cudart().cudaProfilerStop()
    clocks = sampler.stop()
    ms, value = job_throughput(ev0.elapsed_time(ev1) / args.steps, world, torch, dev)
    # device time per solve by phase (CUDA events inside the engine, same timed solves)
    phases = {kk: v / args.steps for kk, v in phase_sum.items()}
    phases["other"] = max(0.0, ms - sum(phases.values()))

    # ---------------- dominant kernel: the sketch product, timed alone.  The engine times
    # each product with CUDA events on its own stream (rsvdpack_last_timing().sketch_ms).
    # Mixed modes: the solve's A X products read a BF16 copy of A (made once per solve) and its
    # A^T X products read the FP32 A through kind::tf32 (TF32 mode) or the BF16 copy (BF16
    # mode); both forms are timed here on the same resident operands.
    X = torch.randn(l, n, device=dev, dtype=tdt)     # column-major n x l
    Y = torch.empty(l, m, device=dev, dtype=tdt)
    Xt = torch.randn(l, m, device=dev, dtype=tdt)
    Z = torch.empty(l, n, device=dev, dtype=tdt)
    mixed = args.precision in ("tf32", "bf16")
    Abf = At.to(torch.bfloat16) if mixed else None
    forms = {}
    for name, trans, (x, ldx, y, ldy) in (("A*X", 0, (X, n, Y, m)), ("A^T*X", 1, (Xt, m, Z, n))):
        if mixed and (trans == 0 or args.precision == "bf16"):
            a_ptr, a_dt, a_es, kname = Abf.data_ptr(), 2, 2, "bf16 (kind::f16)"
        else:
            a_ptr, a_dt, a_es = dA, dt, (8 if dt == 0 else 4)
            kname = "tf32 (kind::tf32)" if mixed else ("fp64 CUDA-core" if dt == 0 else "fp32 CUDA-core")
        x_es = 2 if a_dt == 2 else a_es
        times = []
        for i in range(7):
            rc = L.rsvdpack_dev_sketch(a_ptr, a_dt, m, m, n, x.data_ptr(), ldx, l, y.data_ptr(), ldy, trans)
            if rc:
                raise RuntimeError(f"sketch failed: {eng.last_error()}")
            if i >= 2:
                times.append(eng.last_timing().sketch_ms)
        ms_k = sum(times) / len(times)
        xr, yr = (m, n) if trans else (n, m)
        nbytes = m * n * a_es + xr * l * x_es + yr * l * (8 if dt == 0 else 4)
        forms[name] = {"ms": ms_k, "operand": kname, "bytes": nbytes, "gbs": nbytes / ms_k / 1e6,
                       "tflops": 2.0 * m * n * l / ms_k / 1e9}
    del X, Y, Xt, Z, Abf
    hbm_peak, tc_peak, peak_kind = measured_peaks()
    tot_bytes = sum(f["bytes"] for f in forms.values())
    tot_ms = sum(f["ms"] for f in forms.values())
    gbs = tot_bytes / tot_ms / 1e6
    roof = {"bound": "hbm", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
            "traffic": TC_TRAFFIC_PER_LAUNCH if mixed else None, "peak_kind": peak_kind,
            "kernel": "sketch product " + ("(tcgen05, one A*X and one A^T*X launch)" if mixed else "(CUDA-core GEMM)"),
            "tflops": 2.0 * m * n * l * len(forms) / tot_ms / 1e9, "tensor_peak_tflops": tc_peak, "forms": forms,
            "solve_phases_ms": phases}
    # the whole solve against its own roofline (A's FP32 bytes per pass; the TF32 dense rate
    # taken as half the measured BF16 rate)
    roof["solve"] = (solve_roofline(m, n, k, l, Q, S_ORTH, VNUM, 4, ms, hbm_peak,
                                    tc_peak / 2.0 if args.precision == "tf32" else tc_peak)
                     if mixed else None)

    # ---------------- the plain FP32 GPU form of the same method (CUDA-core GEMMs, no
    # tensor cores), same matrix and sizes: the comparison point for the mixed modes
    plain = None
    if mixed and not args.no_plain:
        eng.set_precision("fp32")
        for _ in range(2):
            solve()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(3):
            solve()
        e1.record(stream)
        e1.synchronize()
        ms_plain = e0.elapsed_time(e1) / 3
        res_plain = residual()
        eng.set_precision(args.precision)
        plain = {"precision": "fp32", "value": 1000.0 / ms_plain, "ms_per_step": ms_plain,
                 "rel_frobenius": res_plain, "speedup_of_value": ms_plain / ms}

    # ---------------- the same solve in BF16 mode (both product forms on the BF16 copy of A),
    # with its own matched-error check against the same FP64 residual
    bf16_leg = None
    if args.precision == "tf32" and not args.no_plain:
        eng.set_precision("bf16")
        L.rsvdpack_reset_omega_counter()
        solve()
        res_bf16 = residual()
        for _ in range(2):
            solve()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(5):
            solve()
        e1.record(stream)
        e1.synchronize()
        ms_bf16 = e0.elapsed_time(e1) / 5
        eng.set_precision(args.precision)
        bf16_leg = {"value": 1000.0 / ms_bf16, "ms_per_step": ms_bf16, "rel_frobenius": res_bf16,
                    "matched": (res_fp64 is None) or (res_bf16 <= (1 + 1e-3) * res_fp64)}

    # ---------------- end to end through the reference C API, pinned host FP64 A
    e2e = None
    if not args.no_e2e:
        A_pin = torch.empty(n, m, dtype=torch.float64, pin_memory=True)   # column-major m x n
        A_pin.copy_(At.double().cpu())
        from lowrankmatrixdecompositioncodes_gb300.capi import Mat
        Mh = Mat(m, n, C.cast(C.c_void_p(A_pin.data_ptr()), C.POINTER(C.c_double)))
        t_e2e = []
        for i in range(args.warmup + args.steps):
            Uo, So, Vo, fr = PMat(), PMat(), PMat(), C.c_int(0)
            t0 = time.perf_counter()
            L.low_rank_svd_rand_decomp_fixed_rank(C.byref(Mh), k, P, VNUM, Q, S_ORTH, C.byref(fr), C.byref(Uo),
                                                  C.byref(So), C.byref(Vo))
            t1 = time.perf_counter()
            eng.check()
            for x in (Uo, So, Vo):
                L.matrix_delete(x)
            if i >= args.warmup:
                t_e2e.append(t1 - t0)
        sec = sum(t_e2e) / len(t_e2e)
        e2e = {"value": world / sec, "unit": "solves/s", "h2d_bytes_per_step": m * n * 8,
               "d2h_bytes_per_step": 8 * (m * k + n * k + k), "ms_per_step": 1000 * sec}
        del A_pin
        # the same call through the float-data ABI of the oneAPI variant (librsvdpack_f32.so,
        # a float host matrix, the same precision mode): half the bytes over the host link
        from lowrankmatrixdecompositioncodes_gb300 import load_engine_f32
        from lowrankmatrixdecompositioncodes_gb300.capi import MatF32
        ef = load_engine_f32()
        ef.set_precision(args.precision)
        ef.set_use_provider(False)
        A_f = torch.empty(n, m, dtype=torch.float32, pin_memory=True)
        A_f.copy_(At.cpu())
        Mf = MatF32(m, n, C.cast(C.c_void_p(A_f.data_ptr()), C.POINTER(C.c_float)))
        t_f = []
        for i in range(args.warmup + args.steps):
            Uo, So, Vo, fr = ef.PMat(), ef.PMat(), ef.PMat(), C.c_int64(0)
            t0 = time.perf_counter()
            ef.lib.low_rank_svd_rand_decomp_fixed_rank(C.byref(Mf), k, P, VNUM, Q, S_ORTH, C.byref(fr), C.byref(Uo),
                                                       C.byref(So), C.byref(Vo))
            t1 = time.perf_counter()
            ef.check()
            for x in (Uo, So, Vo):
                ef.lib.matrix_delete(x)
            if i >= args.warmup:
                t_f.append(t1 - t0)
        sec_f = sum(t_f) / len(t_f)
        e2e["float_abi"] = {"value": world / sec_f, "unit": "solves/s", "h2d_bytes_per_step": m * n * 4,
                            "d2h_bytes_per_step": 4 * (m * k + n * k + k), "ms_per_step": 1000 * sec_f,
                            "library": "librsvdpack_f32.so (oneAPI variant ABI: float data, int64_t dims)"}
        del A_f

    # ---------------- extra legs: each runs on rank 0, and a failure is recorded in the line
    # (as {"error": ...}) instead of ending the run
    def extra(fn, *a, **kw):
        try:
            return fn(*a, **kw)
        except Exception as e:            # the headline line must still be printed
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
            return {"error": f"{type(e).__name__}: {e}"}
        finally:
            eng.set_precision(args.precision)
            eng.set_learned(False)
            eng.set_use_provider(False)

    # learned fixed-precision QB against the plain loop
    learned_leg = None
    if rank == 0 and not args.no_learned and os.path.exists(WEIGHTS):
        eng.load_proposal_model(WEIGHTS)
        learned_leg = extra(learned_qb_leg, torch, eng, dev, profile=(args.profile_leg == "learned"))

    # batched workload
    batched = None
    if rank == 0 and not args.no_batched:
        batched = extra(batched_leg, torch, eng, dev, profile=(args.profile_leg == "batched"))

    # the plain fixed-rank workload (2000 x 1000 FP64) and the two-sided ID / CUR workload
    # (20000 x 10000), each with its oracle check
    c1 = c5 = None
    if rank == 0 and not args.no_c1:
        c1 = extra(plain_fixed_rank_leg, torch, eng)
    if rank == 0 and not args.no_c5:
        c5 = extra(id_cur_leg, torch, eng)

    # ---------------- CPU baseline: the oracle on the host cores, one full solve
    cpu = None
    if rank == 0 and not args.no_cpu:
        A_host = At.T.double().cpu().numpy()
        threads = os.cpu_count() or 1
        t_cpu = cpu_solve_seconds(A_host, threads, repeats=1)
        cpu = {"value": 1.0 / t_cpu[0], "unit": "solves/s", "cores": threads, "kind": "port",
               "sample": "1 full solve of the workload on the CPU oracle (reference algorithm, OpenBLAS)"}
        # one core: the oracle with one OpenMP / BLAS thread, pinned to one core (stands in for the
        # reference's single-core GSL build, which has no fixed-rank routine and no GSL here)
        prev = os.sched_getaffinity(0)
        try:
            os.sched_setaffinity(0, {min(prev)})
            t1 = cpu_solve_seconds(A_host, 1, repeats=1)
        finally:
            os.sched_setaffinity(0, prev)
        cpu["single_core"] = {"value": 1.0 / t1[0], "unit": "solves/s", "cores": 1, "kind": "port",
                              "sample": "1 full solve, 1 thread pinned to one core"}
        del A_host

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            # tf32 mode: A^T X on kind::tf32 from the FP32 A, A X on kind::f16 from A's BF16 copy (the
            # tensor cores read 32-bit operands K-major only); the l x l steps FP32 refined to FP64
            "vs_baseline": None, "dtype": {"fp64": "f64", "fp32": "f32", "tf32": "tf32+bf16", "bf16": "bf16"}[args.precision],
            "data": "synthetic (seeded; A = U diag(i^-1.5) V^T + 1e-4 G)",
            "config": {"workload": "single large rSVD 16384x8192 k=256 p=16 q=2 s=1 vnum=1", "m": m, "n": n, "k": k,
                       "p": P, "q": Q, "s": S_ORTH, "precision": args.precision,
                       "l2": "inputs larger than L2 (A = 512 MiB)", "parallelism": f"replicas x{world}"},
            "residual": {"rel_frobenius": res_mixed, "fp64_same_method": res_fp64,
                         "rel_frobenius_engine_reporter": fro_m / fro_a,
                         "rel_spectral": spec_m / float(sv_lapack[0]),
                         "fp64_same_method_rel_spectral": (spec_fp64 / float(sv_lapack[0])
                                                           if spec_fp64 is not None else None),
                         "sigma_rel_err_topk": sig_mixed, "fp64_same_method_sigma_rel_err_topk": sig_fp64,
                         "sigma_rel_err_top16": sig_mixed16, "fp64_same_method_sigma_rel_err_top16": sig_fp64_16,
                         "sigma_rel_err_mean_topk": sig_mixed_mean,
                         "fp64_same_method_sigma_rel_err_mean_topk": sig_fp64_mean,
                         "sigma_checker": "FP64 LAPACK: top-k eigenvalues of A^T A (dsyevr), square-rooted",
                         "matched": (res_fp64 is None) or (res_mixed <= (1 + 1e-3) * res_fp64),
                         "matched_sigma_rule": "max top-k relative sigma error within 1% of the FP64 path's",
                         "matched_sigma": (sig_fp64 is None) or (sig_mixed <= (1 + 1e-2) * sig_fp64 + 1e-9)},
            "roofline": roof, "plain_gpu": plain, "bf16": bf16_leg, "learned_qb": learned_leg, "batched": batched,
            "plain_fixed_rank_2000x1000": c1, "id_cur_20000x10000": c5,
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clocks,
            "device": name,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0

# ------------------------------------------------------------------ ncu profiling cases
# ``python bench.py --profile-case NAME`` runs one kernel family of the engine on a fixed case:
# warm-up calls first, then exactly one call bracketed by cudaProfilerStart / cudaProfilerStop
# (capture with ``ncu --profile-from-start off``).  Sizes keep the device footprint to a few GB
# and the operands larger than L2 (129 MB), so DRAM counters stay meaningful.
#   update   C (8192 x 16384) -= A^T X, K = 256   (blocked-QB deflation, rsvdpack_dev_update_3xtf32)
#   gemm3x   D (16384 x 256) = A^T X, K = 16384   (B = Q^T A of the block loop, rsvdpack_dev_gemm_3xtf32)
#   solve    one fixed-rank TF32 solve, 16384 x 8192, k = 256, p = 16, q = 2
#   pivot    pivotedQR_mkl of a 520 x 10000 FP64 matrix through the C API (the row sketch of the
#            two-sided ID / CUR workload)
#   norm     the Frobenius-norm sweep of the plain FP32 blocked QB (one block) on a 32768 x 16384
#            FP32 matrix (2 GiB)
#   df64     a reduced sketch pass of the two-sided ID workload as a double-float FP64 product
#            (520 x 8000 by 8000 x 4000, rsvdpack_dev_gemm_df64)
#   lxl      the FP32 l x l Jacobi SVD (rsvdpack_dev_small_svd(..., 1)) of a 272 x 272 factor shaped
#            like the headline workload's: 13 separated singular values i^-1.5, then 259 packed into
#            [0.0166, 0.0218], as the transposed triangular factor the engine hands the Jacobi

def _prof_engine():
    from lowrankmatrixdecompositioncodes_gb300 import load_engine
    eng = load_engine()
    sms, _, cc = eng.device_info()
    if sms <= 0 or cc != (10, 3):
        raise RuntimeError(f"no GB300 visible: {eng.last_error()}")
    return eng


def _prof_run(torch, fn, warm=2):
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()
    fn()
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStop()


def prof_case_update(torch, eng):
    L = eng.lib
    L.rsvdpack_dev_update_3xtf32.argtypes = [C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong, C.c_int, C.c_int,
                                             C.c_int, C.c_void_p, C.c_longlong, C.POINTER(C.c_double)]
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    M, N, K = 8192, 16384, 256
    A = torch.randn(M, K, device="cuda", generator=g)       # K x M column-major
    X = torch.randn(N, K, device="cuda", generator=g)       # K x N column-major
    Cm = torch.randn(N, M, device="cuda", generator=g)      # M x N column-major
    f2 = C.c_double(0)

    def call():
        if L.rsvdpack_dev_update_3xtf32(A.data_ptr(), K, X.data_ptr(), K, M, N, K, Cm.data_ptr(), M, C.byref(f2)):
            raise RuntimeError(eng.last_error())
    _prof_run(torch, call)


def prof_case_gemm3x(torch, eng):
    L = eng.lib
    L.rsvdpack_dev_gemm_3xtf32.argtypes = [C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong, C.c_int, C.c_int,
                                           C.c_int, C.c_void_p, C.c_longlong]
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    M, N, K = 16384, 256, 16384
    A = torch.randn(M, K, device="cuda", generator=g)
    X = torch.randn(N, K, device="cuda", generator=g)
    D = torch.empty(N, M, device="cuda")

    def call():
        if L.rsvdpack_dev_gemm_3xtf32(A.data_ptr(), K, X.data_ptr(), K, M, N, K, D.data_ptr(), M):
            raise RuntimeError(eng.last_error())
    _prof_run(torch, call)


def prof_case_solve(torch, eng):
    L = eng.lib
    L.rsvdpack_dev_svd_fixed_rank.restype = C.c_int
    L.rsvdpack_dev_svd_fixed_rank.argtypes = [C.c_void_p, C.c_int, C.c_longlong, C.c_int, C.c_int, C.c_int, C.c_int,
                                              C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p,
                                              C.c_void_p, C.c_longlong]
    eng.set_precision("tf32")
    eng.set_use_provider(False)
    m, n, k, p = 16384, 8192, 256, 16
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    U0, _ = torch.linalg.qr(torch.randn(m, n, device="cuda", generator=g))
    V0, _ = torch.linalg.qr(torch.randn(n, n, device="cuda", generator=g))
    s = torch.arange(1, n + 1, device="cuda", dtype=torch.float32) ** -1.5
    At = ((U0 * s) @ V0.T + 1e-4 * torch.randn(m, n, device="cuda", generator=g)).T.contiguous()
    torch.backends.cuda.matmul.allow_tf32 = prev
    del U0, V0
    U = torch.empty(k, m, device="cuda")
    V = torch.empty(k, n, device="cuda")
    S = torch.empty(k, device="cuda", dtype=torch.float64)

    def call():
        if L.rsvdpack_dev_svd_fixed_rank(At.data_ptr(), 1, m, m, n, k, p, 1, 2, 1, U.data_ptr(), m, S.data_ptr(),
                                         V.data_ptr(), n):
            raise RuntimeError(eng.last_error())
    _prof_run(torch, call)


def prof_case_pivot(torch, eng):
    import numpy as np
    eng.set_precision("fp64")
    A = np.random.default_rng(2).standard_normal((520, 10000))

    def call():
        eng.pivotedQR_mkl(A)
        eng.check()
    _prof_run(torch, call, warm=1)


def prof_case_norm(torch, eng):
    L = eng.lib
    L.rsvdpack_dev_qb.restype = C.c_int
    L.rsvdpack_dev_qb.argtypes = [C.c_void_p, C.c_int, C.c_longlong, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                  C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong, C.c_int,
                                  C.POINTER(C.c_int)]
    eng.set_precision("fp32")
    eng.set_learned(False)
    m, n, cap = 32768, 16384, 64
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    At = torch.randn(n, m, device="cuda", generator=g)
    Q = torch.empty(cap, m, device="cuda")
    B = torch.empty(n, cap, device="cuda")
    tol = 0.999 * float(torch.linalg.norm(At.double()))           # stops after the first block
    fr = C.c_int(0)

    def call():
        if L.rsvdpack_dev_qb(At.data_ptr(), 1, m, m, n, 64, 0, tol, 1, 1, Q.data_ptr(), m, B.data_ptr(), cap, cap,
                             C.byref(fr)):
            raise RuntimeError(eng.last_error())
    _prof_run(torch, call)


def prof_case_df64(torch, eng):
    """A reduced sketch pass of the two-sided ID workload as a double-float FP64 product:
    Y^T (520 x 4000) = Om (520 x 8000) A (8000 x 4000) (A and its split: 512 MB, above L2)."""
    L = eng.lib
    L.rsvdpack_dev_gemm_df64.restype = C.c_int
    L.rsvdpack_dev_gemm_df64.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_void_p,
                                         C.c_longlong, C.c_void_p, C.c_longlong, C.c_double, C.c_void_p,
                                         C.c_longlong]
    g = torch.Generator(device="cuda")
    g.manual_seed(4)
    M, N, K = 520, 4000, 8000
    Om = torch.randn(M, K, device="cuda", dtype=torch.float64, generator=g)   # K x M column-major
    A = torch.randn(N, K, device="cuda", dtype=torch.float64, generator=g)    # K x N column-major
    Y = torch.empty(N, M, device="cuda", dtype=torch.float64)

    def call():
        if L.rsvdpack_dev_gemm_df64(1, 0, M, N, K, 1.0, Om.data_ptr(), K, A.data_ptr(), K, 0.0, Y.data_ptr(), M):
            raise RuntimeError(eng.last_error())
    _prof_run(torch, call)


def prof_case_lxl(torch, eng):
    import numpy as np
    L = eng.lib
    L.rsvdpack_dev_small_svd.restype = C.c_int
    L.rsvdpack_dev_small_svd.argtypes = [C.c_void_p, C.c_int, C.c_longlong, C.c_void_p, C.c_longlong, C.c_void_p,
                                         C.c_void_p, C.c_longlong, C.c_int]
    n = 272
    g = np.random.default_rng(0)
    head = np.arange(1, 14) ** -1.5
    tail = np.sort(0.0166 + 0.0052 * g.beta(1.3, 1.0, n - 13))[::-1]
    sv = np.concatenate([head, tail])
    Q1, _ = np.linalg.qr(g.standard_normal((n, n)))
    Q2, _ = np.linalg.qr(g.standard_normal((n, n)))
    X = np.linalg.qr((Q1 * sv) @ Q2.T, mode="r").T            # lower triangular: R^T
    G0 = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()    # column-major X
    U = torch.empty(n, n, device="cuda", dtype=torch.float64)
    V = torch.empty_like(U)
    S = torch.empty(n, device="cuda", dtype=torch.float64)

    def call():
        G = G0.clone()
        if L.rsvdpack_dev_small_svd(G.data_ptr(), n, n, U.data_ptr(), n, S.data_ptr(), V.data_ptr(), n, 1) < 0:
            raise RuntimeError(eng.last_error())
    _prof_run(torch, call)


PROFILE_CASES = {"update": prof_case_update, "gemm3x": prof_case_gemm3x, "solve": prof_case_solve,
                 "pivot": prof_case_pivot, "norm": prof_case_norm, "df64": prof_case_df64, "lxl": prof_case_lxl}


def main():
    args = parse()
    if args.profile_case:
        import torch
        PROFILE_CASES[args.profile_case](torch, _prof_engine())
        print("ok", args.profile_case)
        return 0
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
