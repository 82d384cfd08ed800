"""Build librsvdpack.so in-tree with nvcc for sm_103a (GB300).

Each translation unit in csrc/ is compiled in parallel into _build/, then linked into
lowrankmatrixdecompositioncodes_gb300/librsvdpack.so (static CUDA runtime, no libcuda
link-time dependency: the driver API is reached through cudaGetDriverEntryPoint).
api.cu, the reference API layer, is compiled twice more and linked with the same engine
objects: with RSVDPACK_INDEX64 into librsvdpack64.so (int64_t dimensions, as
multi_core_mkl_code_64bit) and with RSVDPACK_REAL32 into librsvdpack_f32.so (float data and
int64_t dimensions, as oneapi_code), over the same kernels.
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
LIBF32 = os.path.join(PKG, "librsvdpack_f32.so")
API_UNIT = "api.cu"
# library -> (object suffix, defines) of its API unit; the other units are shared
VARIANTS = {LIB: ("", ()), LIB64: (".i64", ("-DRSVDPACK_INDEX64",)), LIBF32: (".f32", ("-DRSVDPACK_REAL32",))}
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
    shared = []
    api_objs = {}
    for s in srcs:
        base = os.path.basename(s)
        if base == API_UNIT:
            units = [(lib, os.path.join(BUILD, base + suf + ".o"), extra) for lib, (suf, extra) in VARIANTS.items()]
        else:
            units = [(None, os.path.join(BUILD, base + ".o"), ())]
        for lib, o, extra in units:
            if lib is None:
                shared.append(o)
            else:
                api_objs[lib] = o
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
    for lib in VARIANTS:
        lobjs = shared + [api_objs[lib]]
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
