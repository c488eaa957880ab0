"""The C++ face (include/als_model.hpp): a program written like the reference's main.cpp, compiled
with g++ against the library.  On a machine without a GPU it must fail loudly (NO_DEVICE) after
loading the .bin files; on the GPU it must train the toy sets to the oracle's factors and write
the same libmf model as the Python face."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

import cuda_als_gb300 as ca
from oracle import oracle as O

ROOT = Path(__file__).resolve().parent.parent
LIBDIR = ROOT / "cuda_als_gb300"


@pytest.fixture(scope="module")
def shim_exe(tmp_path_factory):
    out = tmp_path_factory.mktemp("shim") / "shim_main"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror",
           f"-I{ROOT / 'include'}", str(ROOT / "tests" / "cpp" / "shim_main.cpp"), "-o", str(out),
           f"-L{LIBDIR}", "-lals_gb300", f"-Wl,-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _args(tmp_path, toy, f, solve, vtvs=0, out=None):
    from test_abi import _write_dataset

    _write_dataset(tmp_path, toy)
    a = [str(tmp_path), str(toy["m"]), str(toy["n"]), str(len(toy["R_train_csr_data"])),
         str(len(toy["R_test_coo_data"])), str(f), "0.05", "10", str(vtvs), str(solve)]
    return a + ([str(out)] if out else [])


def _has_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device path")
def test_cpp_shim_fails_loudly_without_a_gpu(shim_exe, tmp_path, toy):
    r = subprocess.run([str(shim_exe)] + _args(tmp_path, toy, 8, 0), capture_output=True,
                       text=True)
    assert r.returncode == 3, r.stdout + r.stderr
    assert "ERROR ALS_ERR_NO_DEVICE" in r.stdout


@pytest.mark.gpu
def test_cpp_shim_rejects_wrong_file_size(shim_exe, tmp_path, toy):
    """(GPU only: without a device the first page-locked allocation already fails.)"""
    args = _args(tmp_path, toy, 8, 0)
    args[3] = str(len(toy["R_train_csr_data"]) + 1)  # nnz_train that does not match the files
    r = subprocess.run([str(shim_exe)] + args, capture_output=True, text=True)
    assert r.returncode == 3 and "ERROR ALS_ERR_IO" in r.stdout, r.stdout + r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("solve", [0, 3])
def test_cpp_shim_trains_like_the_oracle(shim_exe, tmp_path, toy, solve):
    f = 100 if toy["m"] == 15 else 20   # config/toy_data.ini, config/toy_data_2.ini
    model_path = tmp_path / "shim.model"
    r = subprocess.run([str(shim_exe)] + _args(tmp_path, toy, f, solve, out=model_path),
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    got = dict(line.split() for line in r.stdout.strip().splitlines())
    m, n = toy["m"], toy["n"]
    csr = (toy["R_train_csr_indptr"], toy["R_train_csr_indices"], toy["R_train_csr_data"])
    csc = (toy["R_train_csc_indptr"], toy["R_train_csc_indices"], toy["R_train_csc_data"])
    Ue, Ve, _ = O.train(m, n, f, 0.05, 10, csr, csc, solve=O.LU if solve == 0 else O.CHOLESKY)
    test = (toy["R_test_coo_row"], toy["R_test_coo_col"], toy["R_test_coo_data"])
    assert abs(float(got["rmse_test"]) - O.rmse(*test, Ue, Ve)) < 1e-4
    raw = model_path.read_bytes()
    assert list(np.frombuffer(raw[:16], np.int32)) == [0, m, n, f]
    body = np.frombuffer(raw[20:], np.float32)
    U, V = body[:m * f].reshape(m, f), body[m * f:].reshape(n, f)
    assert np.linalg.norm(U - Ue) / np.linalg.norm(Ue) < 1e-4
    assert np.linalg.norm(V - Ve) / np.linalg.norm(Ve) < 1e-4
    assert float(got["U0"]) == pytest.approx(float(U[0, 0]), rel=1e-6)
    assert got["solve"] == ("LU" if solve == 0 else "CHOLESKY")
