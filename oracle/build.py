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


if __name__ == "__main__":
    print(build(verbose=True))
