"""Build libals_gb300.so in-tree with nvcc for sm_103a (no torch, no cmake).

Each translation unit compiles in parallel; the shared object is re-linked only when a source
or header is newer than it.  Host code is plain C++17 (portable between x86-64 and aarch64).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
OBJDIR = PKG / "_build" / platform.machine()  # x86-64 here, aarch64 on the GPU machine
LIB = PKG / "libals_gb300.so"
CLI = PKG / "als_gb300_main"

SOURCES = [
    "api.cpp",
    "eventlog.cpp",
    "sweep.cpp",
    "synth.cpp",
    "index_kernels.cu",
    "coo_build.cu",
    "init.cu",
    "sweep_fp32.cu",
    "sweep_tc.cu",
    "sweep_tc_fp32.cu",
    "sweep_tc_fp64.cu",
    "sweep_tc_fp112.cu",
    "sweep_tc_fp128.cu",
    "sweep_tc_fp32_e4m3.cu",
    "sweep_tc_fp64_e4m3.cu",
    "sweep_tc_fp112_e4m3.cu",
    "sweep_tc_fp128_e4m3.cu",
    "rmse.cu",
    "adjoint.cu",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp,-O3",
          "-Xcompiler", "-Wall,-Wno-unused-function"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libals_gb300")


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(target: Path, inputs: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(p.stat().st_mtime > t for p in inputs)


def _compile(src: str, extra: list[str], verbose: bool) -> Path:
    obj = OBJDIR / (src.replace(".", "_") + ".o")
    if _stale(obj, [CSRC / src] + _deps()):
        cmd = [nvcc(), "-c", str(CSRC / src), "-o", str(obj), *ARCH, *CFLAGS, *extra]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, flush=True)
    return obj


def build(verbose: bool = False, ptxas_info: bool = False) -> Path:
    """Compile every translation unit for sm_103a and link libals_gb300.so in the package."""
    OBJDIR.mkdir(parents=True, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    srcs = [s for s in SOURCES if (CSRC / s).exists()]
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, verbose or ptxas_info), srcs))
    stamp = OBJDIR / "linked"
    if _stale(LIB, objs) or _stale(stamp, objs) or _stale(stamp, [LIB]):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), "-shared", "-o", str(tmp), *map(str, objs), *ARCH,
               "-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
        stamp.touch()
    build_cli(verbose)
    return LIB


def build_cli(verbose: bool = False) -> Path:
    """The command-line driver (csrc/als_main.cpp, host C++ over the C ABI) next to the library."""
    src = CSRC / "als_main.cpp"
    if _stale(CLI, [src, LIB] + sorted(INCLUDE.glob("*.hpp")) + sorted(INCLUDE.glob("*.h"))):
        cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
        tmp = CLI.with_suffix(".tmp")
        cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Wextra", f"-I{INCLUDE}", str(src), "-o",
               str(tmp), f"-L{PKG}", "-lals_gb300", "-Wl,-rpath,$ORIGIN"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"building {CLI.name} failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, CLI)
    return CLI


if __name__ == "__main__":
    import sys

    print(build(verbose=True, ptxas_info="-v" in sys.argv))
