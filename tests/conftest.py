"""Shared test fixtures.

Libraries under test:
  * ``engine``  -- the GPU engine, librsvdpack.so (the product; needs a GPU to compute,
                   loads and exports its symbols without one);
  * ``port``    -- oracle/port/librsvd_port.so, the CPU restatement (test oracle);
  * ``ref``     -- oracle/_ref/librsvd_ref.so, the reference's own sources built by
                   ``make -C oracle ref`` (only where the reference tree exists).
All three export the reference's C API, so one binding (capi.RsvdLibrary) drives them.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

# the batched path's autotuner keeps its table in a file: a fresh one for every test session
os.environ.setdefault("RSVDPACK_TUNE_FILE", os.path.join(tempfile.gettempdir(),
                                                         f"rsvdpack_batch_tune_{os.getpid()}.txt"))

GOLDEN = os.path.join(ROOT, "tests", "golden")
PORT_SO = os.path.join(ROOT, "oracle", "port", "librsvd_port.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "librsvd_ref.so")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


def _gpu_available() -> bool:
    try:
        from lowrankmatrixdecompositioncodes_gb300 import engine_available
        return engine_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _gpu_available():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU visible")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def port():
    from lowrankmatrixdecompositioncodes_gb300.capi import RsvdLibrary
    if not os.path.exists(PORT_SO):
        subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"])
    return RsvdLibrary(PORT_SO)


@pytest.fixture(scope="session")
def ref():
    from lowrankmatrixdecompositioncodes_gb300.capi import RsvdLibrary
    if not os.path.exists(REF_SO):
        pytest.skip("reference build (oracle/_ref) not present on this machine")
    return RsvdLibrary(REF_SO)


@pytest.fixture(scope="session")
def engine():
    from lowrankmatrixdecompositioncodes_gb300 import load_engine
    return load_engine()


def golden_cases():
    with open(os.path.join(GOLDEN, "index.json")) as f:
        return json.load(f)


def load_golden(key):
    meta = golden_cases()[key]
    z = np.load(os.path.join(GOLDEN, key + ".npz"))
    A = np.load(os.path.join(GOLDEN, meta["matrix"]))["A"]
    outs = [z[f"out{i}"] for i in range(meta["n_out"])]
    omegas = [z[f"omega{i}"] for i in range(meta["n_omega"])]
    return meta, A, outs, omegas


def spectrum_matrix(m, n, s, seed):
    g = np.random.default_rng(seed)
    r = min(m, n)
    U, _ = np.linalg.qr(g.standard_normal((m, r)))
    V, _ = np.linalg.qr(g.standard_normal((n, r)))
    return (U * s[:r]) @ V.T
