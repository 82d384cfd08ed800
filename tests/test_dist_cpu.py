"""The multi-rank path of bench.py on the CPU (gloo, world size 2, 127.0.0.1): the job's
throughput comes from the slowest rank's time (MAX over ranks), and the reference arm runs on
rank 0 only -- the other ranks exit 0 without work or output."""
import os
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, value = bench.job_throughput(10.0 + 5.0 * rank, world, torch, "cpu")
    q.put((rank, ms, value))
    dist.destroy_process_group()


def test_job_throughput_takes_the_slowest_rank():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, value in got:
        assert ms == 15.0                                  # max over ranks
        assert abs(value - 2 * 1000.0 / 15.0) < 1e-9       # whole-job rate


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr[-500:]
    assert r.stdout.strip() == ""


def test_solve_roofline_of_the_headline_workload():
    """The whole-solve roofline bench.py reports: 16384 x 8192, l = 272, q = 2 (4 passes over A),
    s = 1, vnum = 1 (four orthonormalisations), FP32 A, the measured peaks of the pool."""
    import bench
    r = bench.solve_roofline(16384, 8192, 256, 272, 2, 1, 1, 4, 5.35, 6791.0, 1935.3 / 2)
    m, n, l, k = 16384, 8192, 272, 256
    want = 4 * 2.0 * m * n * l + 4.0 * l * l * (2 * m + 2 * n) + 22.0 * l ** 3 + 2.0 * (m + n) * l * k
    assert r["passes"] == 4 and abs(r["flops"] - want) < 1e-6 * want
    assert r["bytes"] == 4 * m * n * 4
    assert r["bound"] == "tensor" and 0.3 < r["roofline_ms"] < 0.34
    assert abs(r["frac"] - r["roofline_ms"] / 5.35) < 1e-12
    # q = 3, s = 2: power rounds j = 1, 2 orthonormalise at 2j - 2 = 0, 2 only
    r2 = bench.solve_roofline(1000, 500, 10, 20, 3, 2, 2, 8, 1.0, 6791.0, 1935.3)
    assert r2["passes"] == 6
    assert abs(r2["flops"] - (6 * 2.0 * 1000 * 500 * 20 + 4.0 * 400 * (1000 + 1000 + 1000)
                              + 22.0 * 20 ** 3 + 2.0 * 1500 * 20 * 10)) < 1e-3
