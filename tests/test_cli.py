"""The command-line driver (cuda_als_gb300/als_gb300_main, csrc/als_main.cpp) against the
reference's main.cpp: same INI keys and .bin files, same log lines in the same order
(oracle/eventlog.py's main_calls), test RMSE and libmf model as the FP64 oracle's.

CPU: usage and unreadable-INI exits; without a device the run fails loudly (ALS_ERR_NO_DEVICE)
after writing the parameter line, and the log so far is saved.  GPU: two runs with
per-iteration RMSE lines; one run that saves the model.
"""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

import cuda_als_gb300 as ca
from conftest import ROOT
from oracle import eventlog as E
from oracle import oracle as O

CLI = ROOT / "cuda_als_gb300" / "als_gb300_main"


def _has_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def _setup(tmp_path, toy, runs, iters, solve, iter_rmse, model_path=""):
    from test_abi import _write_dataset

    data = tmp_path / "data"
    data.mkdir()
    _write_dataset(data, toy)
    logdir = tmp_path / "log"
    logdir.mkdir()
    f = 100 if toy["m"] == 15 else 20  # config/toy_data.ini, config/toy_data_2.ini
    nnz, nt = len(toy["R_train_csr_data"]), len(toy["R_test_coo_data"])
    ini = tmp_path / "toy.ini"
    ini.write_text(f"""[general]
log_folder = {logdir}
als_runs = {runs}

[data]
data_folder = {data}
m = {toy['m']}
n = {toy['n']}
nnz_train = {nnz}
nnz_test = {nt}

[als]
f = {f}
lambda = 0.05
als_iters = {iters}
als_calculate_vtvs_type = 1
als_solve_type = {solve}
m_batches = 1
n_batches = 1

[als_gb300]
iter_rmse = {int(iter_rmse)}
model_path = {model_path}
""")
    params = E.params_text(toy["m"], toy["n"], f, nnz, nt, 0.05, iters, str(data), runs,
                           str(logdir), 1, solve)
    return ini, logdir, f, params


def _run(*args):
    return subprocess.run([str(CLI), *map(str, args)], capture_output=True, text=True, timeout=300)


def test_cli_usage_and_unreadable_ini(tmp_path):
    assert CLI.exists()
    r = _run()
    assert r.returncode == 2 and "usage" in r.stderr
    r = _run(tmp_path / "missing.ini")
    assert r.returncode == 1 and r.stdout.startswith("Can't load ")


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device path")
def test_cli_fails_loudly_without_a_gpu_and_keeps_the_log(tmp_path, toy):
    ini, logdir, _, params = _setup(tmp_path, toy, 1, 2, 0, False)
    r = _run(ini)
    assert r.returncode == 3 and "ERROR ALS_ERR_NO_DEVICE" in r.stdout, r.stdout + r.stderr
    logs = list(logdir.iterdir())
    assert len(logs) == 1 and E.NAME_RE.match(logs[0].name)
    parsed = E.parse(logs[0].read_text())
    assert E.check_columns(parsed) is None
    assert E.rows_of(parsed) == E.expected_rows([("log", params)])


def _split(rows):
    vals, out = [], []
    for (i, r, a, ev, t) in rows:
        for prefix in ("RMSE test: ", "final RMSE test: "):
            if t.startswith(prefix):
                vals.append(float(t[len(prefix):]))
                t = prefix + "{rmse}"
        out.append((i, r, a, ev, t))
    return out, vals


def _oracle(toy, f, iters, solve):
    m, n = toy["m"], toy["n"]
    csr = (toy["R_train_csr_indptr"], toy["R_train_csr_indices"], toy["R_train_csr_data"])
    csc = (toy["R_train_csc_indptr"], toy["R_train_csc_indices"], toy["R_train_csc_data"])
    test = (toy["R_test_coo_row"], toy["R_test_coo_col"], toy["R_test_coo_data"])
    per_iter = []
    for k in range(1, iters + 1):
        U, V, _ = O.train(m, n, f, 0.05, k, csr, csc, solve=solve)
        per_iter.append(O.rmse(*test, U, V))
    return per_iter, U, V


@pytest.mark.gpu
@pytest.mark.parametrize("solve", [0, 3])
def test_cli_two_runs_write_the_reference_log(tmp_path, toy, solve):
    iters = 3
    ini, logdir, f, params = _setup(tmp_path, toy, 2, iters, solve, True)
    r = _run(ini)
    assert r.returncode == 0, r.stdout + r.stderr
    logs = list(logdir.iterdir())
    assert len(logs) == 1
    parsed = E.parse(logs[0].read_text())
    assert E.check_columns(parsed) is None
    got, vals = _split(E.rows_of(parsed))
    exp = E.expected_rows(E.main_calls(params, 2, iters, True, False))
    assert got == exp
    per_iter, _, _ = _oracle(toy, f, iters, O.LU if solve == 0 else O.CHOLESKY)
    want = per_iter * 2  # per run: after iterations 1..iters-1, then the final RMSE
    assert np.allclose(vals, want, atol=2e-4), (vals, want)
    echo, _ = _split([(0,) + x for x in E.echo_rows(r.stdout)])
    assert [x[1:] for x in echo] == [x[1:] for x in exp[1:]]


@pytest.mark.gpu
def test_cli_single_run_saves_the_model(tmp_path, toy):
    iters = 10
    model = tmp_path / "toy.model"
    ini, logdir, f, params = _setup(tmp_path, toy, 1, iters, 3, False, model_path=model)
    r = _run(ini)
    assert r.returncode == 0, r.stdout + r.stderr
    parsed = E.parse(next(logdir.iterdir()).read_text())
    got, vals = _split(E.rows_of(parsed))
    assert got == E.expected_rows(E.main_calls(params, 1, iters, False, True))
    per_iter, Ue, Ve = _oracle(toy, f, iters, O.CHOLESKY)
    assert abs(vals[0] - per_iter[-1]) < 2e-4
    raw = model.read_bytes()
    m, n = toy["m"], toy["n"]
    assert list(np.frombuffer(raw[:16], np.int32)) == [0, m, n, f]
    body = np.frombuffer(raw[20:], np.float32)
    U, V = body[:m * f].reshape(m, f), body[m * f:].reshape(n, f)
    assert np.linalg.norm(U - Ue) / np.linalg.norm(Ue) < 1e-4
    assert np.linalg.norm(V - Ve) / np.linalg.norm(Ve) < 1e-4
    # argv[2] overrides the INI's model_path
    other = tmp_path / "other.model"
    r = _run(ini, other)
    assert r.returncode == 0 and other.read_bytes()[:16] == raw[:16]
