"""Two-sided ID and CUR on the full-size ID/CUR workload: A 20000 x 10000 = U diag(i^-2) V^T
(Haar factors; the spectrum is truncated at rank 1000, where i^-2 is already 1e-6),
k=500, p=20, q=2, s=1, FP64.  The engine and the CPU oracle get the same supplied test
matrix; the column and row index sets must be identical, T / S / C / U / R must agree, and
the CUR residual must match the oracle's."""
import time

import numpy as np
import pytest

from lowrankmatrixdecompositioncodes_gb300.capi import SeededOmega

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

M, N, K, P, Q, S = 20000, 10000, 500, 20, 2, 1


@pytest.fixture(scope="module")
def matrix():
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    r = 1000
    U, _ = torch.linalg.qr(torch.randn(M, r, device="cuda", dtype=torch.float64, generator=g))
    V, _ = torch.linalg.qr(torch.randn(N, r, device="cuda", dtype=torch.float64, generator=g))
    s = torch.arange(1, r + 1, device="cuda", dtype=torch.float64) ** -2.0
    A = ((U * s) @ V.T).cpu().numpy()
    del U, V
    torch.cuda.empty_cache()
    return A


def _run(lib, fn, A, *args):
    lib.set_omega(SeededOmega(2026))
    t0 = time.perf_counter()
    out = getattr(lib, fn)(A, *args)
    return out, time.perf_counter() - t0


def test_two_sided_id_full_size_index_sets_match(engine, port, matrix):
    engine.set_precision("fp64")
    (Ic_o, Ir_o, T_o, S_o), t_cpu = _run(port, "id_two_sided_rand_decomp_fixed_rank", matrix, K, P, Q, S)
    (Ic_e, Ir_e, T_e, S_e), t_gpu = _run(engine, "id_two_sided_rand_decomp_fixed_rank", matrix, K, P, Q, S)
    engine.check()
    print(f"two-sided ID 20000x10000 k=500: oracle {t_cpu:.2f} s, engine {t_gpu:.2f} s")
    assert np.array_equal(Ic_e[:K], Ic_o[:K]), "column index sets differ"
    assert np.array_equal(Ir_e[:K], Ir_o[:K]), "row index sets differ"
    assert np.array_equal(Ic_e, Ic_o) and np.array_equal(Ir_e, Ir_o)
    for got, want in ((T_e, T_o), (S_e, S_o)):
        assert np.max(np.abs(got - want)) / np.max(np.abs(want)) < 1e-6


def test_cur_full_size_matches_oracle(engine, port, matrix):
    engine.set_precision("fp64")
    (C_o, U_o, R_o), t_cpu = _run(port, "cur_rand_decomp_fixed_rank", matrix, K, P, Q, S)
    (C_e, U_e, R_e), t_gpu = _run(engine, "cur_rand_decomp_fixed_rank", matrix, K, P, Q, S)
    engine.check()
    print(f"CUR 20000x10000 k=500: oracle {t_cpu:.2f} s, engine {t_gpu:.2f} s")
    assert np.array_equal(C_e, C_o) and np.array_equal(R_e, R_o)     # exact gathers of the same indices
    Ad = torch.from_numpy(matrix).cuda()
    res = []
    for C_, U_, R_ in ((C_o, U_o, R_o), (C_e, U_e, R_e)):
        Ct, Ut, Rt = (torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (C_, U_, R_))
        res.append(float(torch.linalg.norm(Ad - Ct @ Ut @ Rt) / torch.linalg.norm(Ad)))
    assert res[1] <= res[0] * (1 + 1e-3) + 1e-12, res


def test_two_sided_id_full_size_fp64x(engine, port, matrix):
    """The same workload in the FP64X mode (the sketch passes as double-float products on the
    FP32 pipe): index sets identical to the oracle's."""
    engine.set_precision("fp64x")
    try:
        (Ic_o, Ir_o, T_o, S_o), t_cpu = _run(port, "id_two_sided_rand_decomp_fixed_rank", matrix, K, P, Q, S)
        (Ic_e, Ir_e, T_e, S_e), t_gpu = _run(engine, "id_two_sided_rand_decomp_fixed_rank", matrix, K, P, Q, S)
        engine.check()
        print(f"two-sided ID 20000x10000 k=500 (FP64X): oracle {t_cpu:.2f} s, engine {t_gpu:.2f} s "
              f"(engine call {engine.last_timing().total_ms:.0f} ms)")
    finally:
        engine.set_precision("fp64")
    assert np.array_equal(Ic_e, Ic_o), "column index sets differ"
    assert np.array_equal(Ir_e, Ir_o), "row index sets differ"
    for got, want in ((T_e, T_o), (S_e, S_o)):
        assert np.max(np.abs(got - want)) / np.max(np.abs(want)) < 1e-6
