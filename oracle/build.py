"""Build the oracle (test infrastructure only) into oracle/_build/liboracle.so with gcc -fopenmp.

The oracle is the checker for the CUDA library and the timed CPU baseline; the product never
links or calls it.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / f"liboracle-{platform.machine()}.so"
SRCS = [HERE / "als_oracle.c"]
DEPS = SRCS + [HERE / "als_oracle.h", HERE / "als_oracle_impl.inc"]


def build(verbose: bool = False) -> Path:
    OUT.parent.mkdir(exist_ok=True)
    if OUT.exists() and all(p.stat().st_mtime <= OUT.stat().st_mtime for p in DEPS):
        return OUT
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [cc, "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-Wall",
           *map(str, SRCS), "-o", str(tmp), "-lm"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


# The reference's own logger (logger.cpp, a few hundred lines of standard C++), compiled from
# its sources where they lie, with a call-script driver: the pin of the event-log format.  Only
# where the reference tree is present; the output stays in oracle/_ref/ (git-ignored).
REF_SRC = Path("/root/reference")
REF_OUT = HERE / "_ref" / f"ref_logger-{platform.machine()}"


def build_ref(verbose: bool = False) -> Path | None:
    """Build oracle/_ref/ref_logger from the reference's logger.cpp; None when it is absent."""
    src = REF_SRC / "logger.cpp"
    driver = HERE / "ref_logger_driver.cpp"
    if not src.exists() or not (REF_SRC / "logger.h").exists():
        return REF_OUT if REF_OUT.exists() else None
    deps = [src, REF_SRC / "logger.h", driver]
    if REF_OUT.exists() and all(p.stat().st_mtime <= REF_OUT.stat().st_mtime for p in deps):
        return REF_OUT
    REF_OUT.parent.mkdir(exist_ok=True)
    cxx = os.environ.get("CXX") or shutil.which("g++") or "c++"
    tmp = REF_OUT.with_name(REF_OUT.name + ".tmp")
    cmd = [cxx, "-O2", "-std=c++17", f"-I{REF_SRC}", str(driver), str(src), "-o", str(tmp)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference logger build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, REF_OUT)
    return REF_OUT


if __name__ == "__main__":
    print(build(verbose=True))
    print(build_ref(verbose=True))
