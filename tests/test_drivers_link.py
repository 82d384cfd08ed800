"""The drop-in at the source level: the reference's own driver programs compile unchanged against
the compatibility headers (include/compat/<variant>/, the reference's header names over
rsvdpack.h) and link against the matching library, with no symbol missing -- except randQB_p, the
single-vector QB that multi_core_mkl_code/driver_multi_core_mkl2.c also times (out of scope: not
on the randomized range finder's path).  Needs the reference tree (read-only; each driver is
copied to a temporary directory so that its own directory's headers are not found first) and gcc.
"""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

REF = os.environ.get("RSVDPACK_REFERENCE", "/root/reference")
PKG = os.path.join(ROOT, "lowrankmatrixdecompositioncodes_gb300")
DRIVERS = [
    ("multi_core_mkl_code/driver_multi_core_mkl1.c", "mkl", "rsvdpack"),
    ("multi_core_mkl_code/driver_multi_core_mkl2.c", "mkl", "rsvdpack"),
    ("multi_core_mkl_code/driver_multi_core_mkl3.c", "mkl", "rsvdpack"),
    ("multi_core_mkl_code/driver_multi_core_mkl4.c", "mkl", "rsvdpack"),
    ("multi_core_mkl_code/driver_multi_core_mkl5.c", "mkl", "rsvdpack"),
    ("multi_core_mkl_code_64bit/driver1.c", "mkl64", "rsvdpack64"),
    ("oneapi_code/driver1.c", "oneapi", "rsvdpack_f32"),
    ("oneapi_code/driver2.c", "oneapi", "rsvdpack_f32"),
    ("oneapi_code/driver3.c", "oneapi", "rsvdpack_f32"),
]
OUT_OF_SCOPE = {"multi_core_mkl_code/driver_multi_core_mkl2.c": {"randQB_p"}}


@pytest.mark.parametrize("src,compat,lib", DRIVERS)
def test_reference_driver_links(tmp_path, src, compat, lib):
    path = os.path.join(REF, src)
    if not os.path.exists(path) or shutil.which("gcc") is None:
        pytest.skip("reference tree or gcc not present on this machine")
    if not os.path.exists(os.path.join(PKG, f"lib{lib}.so")):
        pytest.skip("library not built")
    local = tmp_path / os.path.basename(src)
    shutil.copy(path, local)
    cmd = ["gcc", "-w", "-fopenmp", "-I", os.path.join(ROOT, "include", "compat", compat),
           "-I", os.path.join(ROOT, "include"), str(local), f"-L{PKG}", f"-l{lib}", f"-Wl,-rpath,{PKG}",
           "-lm", "-o", str(tmp_path / "driver")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    missing = set()
    for line in r.stderr.splitlines():
        if "undefined reference to `" in line:
            missing.add(line.split("undefined reference to `")[1].rstrip("'"))
    compile_errors = [ln for ln in r.stderr.splitlines() if ": error:" in ln and not ln.startswith("collect2")]
    assert not compile_errors, compile_errors[:5]
    assert missing == OUT_OF_SCOPE.get(src, set()), missing
    if not missing:
        assert r.returncode == 0, r.stderr[-500:]
