"""Build librsvdpack.so in-tree with nvcc for sm_103a (GB300).

Each translation unit in csrc/ is compiled in parallel into _build/, then linked into
lowrankmatrixdecompositioncodes_gb300/librsvdpack.so (static CUDA runtime, no libcuda
link-time dependency: the driver API is reached through cudaGetDriverEntryPoint).
api.cu, the reference API layer, is compiled a second time with RSVDPACK_INDEX64 and linked
with the same engine objects into librsvdpack64.so: the reference API with int64_t
dimensions (multi_core_mkl_code_64bit), over the same kernels.
Incremental: a unit is rebuilt when it or any header in csrc/ or include/ is newer
than its object file.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "librsvdpack.so")
LIB64 = os.path.join(PKG, "librsvdpack64.so")
INDEX64_UNIT = "api.cu"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    for cand in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return [*ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3",
            "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"), "-I", CSRC, *extra]


def _newest_header() -> float:
    hs = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    nvcc = nvcc_path()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr_t = _newest_header()
    todo = []
    objs = []
    objs64 = []
    for s in srcs:
        units = [(os.path.join(BUILD, os.path.basename(s) + ".o"), ())]
        if os.path.basename(s) == INDEX64_UNIT:
            units.append((os.path.join(BUILD, os.path.basename(s) + ".i64.o"), ("-DRSVDPACK_INDEX64",)))
        for o, extra in units:
            if not extra:
                objs.append(o)
            if extra or os.path.basename(s) != INDEX64_UNIT:
                objs64.append(o)
            if not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_t):
                todo.append((s, o, extra))

    def compile_one(soe):
        s, o, extra = soe
        cmd = [nvcc, *_flags(extra), "-c", s, "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(s)}:\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return s

    if todo:
        with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
            for s in ex.map(compile_one, todo):
                if verbose:
                    print("compiled", os.path.basename(s))
    for lib, lobjs in ((LIB, objs), (LIB64, objs64)):
        if todo or not os.path.exists(lib):
            tmp = lib + ".tmp"
            cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *lobjs, "-Xlinker", "-Bsymbolic", "-Xlinker", "--no-undefined"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link of {os.path.basename(lib)} failed:\n{r.stderr}")
            os.replace(tmp, lib)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
