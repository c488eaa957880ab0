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


# The workload generator (the library's synth.cpp, plain C++ with OpenMP) built on its own into
# an oracle-side library, so that the CPU reference arm of the bench generates the same bytes
# without loading the product library.  oracle/synth_errors.cpp stands in for the one library
# function synth.cpp calls (the error recorder).
SYNTH_SRC = HERE.parent / "cuda_als_gb300" / "csrc" / "synth.cpp"
SYNTH_OUT = HERE / "_build" / f"libsynth-{platform.machine()}.so"


def build_synth(verbose: bool = False) -> Path:
    deps = [SYNTH_SRC, HERE / "synth_errors.cpp", SYNTH_SRC.parent / "internal.h",
            HERE.parent / "include" / "als_gb300.h"]
    if SYNTH_OUT.exists() and all(p.stat().st_mtime <= SYNTH_OUT.stat().st_mtime for p in deps):
        return SYNTH_OUT
    SYNTH_OUT.parent.mkdir(exist_ok=True)
    cxx = os.environ.get("CXX") or shutil.which("g++") or "c++"
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda_inc = Path(nvcc).resolve().parent.parent / "include"  # cuda_runtime.h (declarations)
    tmp = SYNTH_OUT.with_suffix(".so.tmp")
    cmd = [cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", f"-I{cuda_inc}",
           str(SYNTH_SRC), str(HERE / "synth_errors.cpp"), "-o", str(tmp)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"generator build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, SYNTH_OUT)
    return SYNTH_OUT


# The reference tree these recipes compile from: $CUDA_ALS_REFERENCE, by default the read-only
# checkout this build was made against.  Absent on machines that only run the prebuilt files.
REF_SRC = Path(os.environ.get("CUDA_ALS_REFERENCE", "/root/reference"))

# The reference's own logger (logger.cpp, a few hundred lines of standard C++), compiled from
# its sources where they lie, with a call-script driver: the pin of the event-log format.  Only
# where the reference tree is present; the output stays in oracle/_ref/ (git-ignored).
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


# The reference's own Gram and CG kernels, compiled from its sources where they lie into
# device-only cubins for sm_103a: `calculate_vtvs` (als_model.cu:91-167, the Gram of its SIMPLE
# vtvs type) and `updateXWithCGKernel` (cumf_als_cg/cg.cu:37-232).  A cubin holds GPU code only,
# so it is built here and loaded on the GPU machine (oracle/refkernels.py), where the reference tree
# is absent.  als_model.cu's host code calls cusparseScsrmm2, which CUDA 11 removed; that call
# is defined away on the command line: it sits in host code that no cubin contains.
REF_CUBINS = {
    "model": (REF_SRC / "als_model.cu", HERE / "_ref" / "ref_model.cubin"),
    "cg": (REF_SRC / "cumf_als_cg" / "cg.cu", HERE / "_ref" / "ref_cg.cubin"),
}


def build_ref_cubins(verbose: bool = False) -> dict[str, Path]:
    """Build oracle/_ref/ref_{model,cg}.cubin where the reference sources are present; return
    the cubins that exist."""
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = {}
    for key, (src, dst) in REF_CUBINS.items():
        if src.exists() and Path(nvcc).exists() and not (
                dst.exists() and src.stat().st_mtime <= dst.stat().st_mtime):
            dst.parent.mkdir(exist_ok=True)
            tmp = dst.with_name(dst.name + ".tmp")
            cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                   f"-I{REF_SRC}", f"-I{REF_SRC / 'cumf_als_cg'}",
                   "-DcusparseScsrmm2(...)=CUSPARSE_STATUS_NOT_SUPPORTED",
                   "-diag-suppress", "177", str(src), "-o", str(tmp)]
            if verbose:
                print(" ".join(cmd), flush=True)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"reference cubin build failed for {src.name}:\n{r.stderr}")
            os.replace(tmp, dst)
        if dst.exists():
            out[key] = dst
    return out


if __name__ == "__main__":
    print(build(verbose=True))
    print(build_synth(verbose=True))
    print(build_ref(verbose=True))
    print(build_ref_cubins(verbose=True))
