"""The event log (als_log_* in include/als_gb300.h, the Python `logger`, include/als_logger.hpp)
against the reference's logger: the CSV columns and their relations, the line order the
reference's main.cpp + als_model::train write, and the stdout echo.

CPU: the oracle's restatement (oracle/eventlog.py) against the CSV and echo the reference's own
logger.cpp wrote for a script of calls (tests/golden/ref_log_script.*); the library's log and the
C++ face replaying that script; the reference's logger live where its sources are present; the
C ABI's argument checks.  GPU: als_train's lines with a log attached (per-iteration events and
test RMSE against the FP64 oracle; results unchanged by logging).
"""
from __future__ import annotations

import subprocess
import time
from pathlib import Path

import numpy as np
import pytest

import cuda_als_gb300 as ca
from conftest import GOLDEN, ROOT
from oracle import build as ob
from oracle import eventlog as E
from oracle import oracle as O

SCRIPT = (GOLDEN / "ref_log_script.txt").read_text()
LIBDIR = ROOT / "cuda_als_gb300"


def _golden_calls():
    import importlib.util

    spec = importlib.util.spec_from_file_location("mlf", GOLDEN / "make_log_fixture.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.script_calls()


def _replay(lg: "ca.logger", script: str):
    """The ref_logger driver's script interpreter (oracle/ref_logger_driver.cpp) on a logger."""
    for line in script.splitlines():
        op, _, rest = line.partition(" ")
        if op == "log":
            c, _, text = rest.partition(" ")
            lg.log(text, c == "1")
        elif op == "start":
            lg.event_started(int(rest))
        elif op == "finish":
            e, c = rest.split()
            lg.event_finished(int(e), c == "1")
        elif op == "iters":
            r, a = rest.split()
            lg.run_iter, lg.als_iter = int(r), int(a)
        elif op == "sleep_us":
            time.sleep(int(rest) * 1e-6)


def _echo_expected(rows):
    return [(r, a, ev, t) for (_, r, a, ev, t) in rows[1:]]


# ---------------------------------------------------------------------------------------------
# The oracle against the reference logger's own output


def test_oracle_matches_the_reference_loggers_csv():
    parsed = E.parse((GOLDEN / "ref_log_script.csv").read_text())
    assert E.check_columns(parsed) is None
    calls = _golden_calls()
    assert E.to_script(calls, write_cout=True, sleep_us=300) == SCRIPT
    assert E.rows_of(parsed) == E.expected_rows(calls)


def test_oracle_matches_the_reference_loggers_echo():
    echo = E.echo_rows((GOLDEN / "ref_log_script.stdout").read_text())
    assert echo == _echo_expected(E.expected_rows(_golden_calls()))


def test_oracle_column_check_catches_a_planted_error():
    parsed = E.parse((GOLDEN / "ref_log_script.csv").read_text())
    bad = [dict(d) for d in parsed]
    k = next(i for i, d in enumerate(bad) if d["event_elapsed"])
    bad[k]["prev_ts"] = bad[k]["curr_ts"]  # an event line that advanced prev_ts
    assert E.check_columns(bad) is not None
    bad = [dict(d) for d in parsed]
    bad[3]["id"] = "7"
    assert E.check_columns(bad) is not None


# ---------------------------------------------------------------------------------------------
# The library's log (host only: no device needed)


def test_library_log_writes_what_the_reference_logger_writes(capfd):
    lg = ca.logger("")
    _replay(lg, SCRIPT)
    parsed = E.parse(lg.text())
    assert E.check_columns(parsed) is None
    assert E.rows_of(parsed) == E.rows_of(E.parse((GOLDEN / "ref_log_script.csv").read_text()))
    assert E.NAME_RE.match(lg.log_name)
    out = capfd.readouterr().out
    assert E.echo_rows(out) == E.echo_rows((GOLDEN / "ref_log_script.stdout").read_text())
    lg.close()


def test_library_log_save_paths(tmp_path):
    lg = ca.logger(str(tmp_path))
    lg.log("one line", False)
    lg.save()  # <log_folder>/<log_name>
    assert (tmp_path / lg.log_name).read_text() == lg.text()
    lg.save(str(tmp_path / "explicit.csv"))
    assert (tmp_path / "explicit.csv").read_text() == lg.text()
    with pytest.raises(ca.ALSError) as e:
        lg.save(str(tmp_path / "no" / "such" / "dir.csv"))
    assert e.value.status == ca.Status.IO
    lg.close()


def test_library_log_argument_checks():
    lg = ca.logger()
    with pytest.raises(ca.ALSError) as e:
        lg.event_started(4)
    assert e.value.status == ca.Status.INVALID_ARG
    with pytest.raises(ca.ALSError):
        lg.event_finished(-1)
    with pytest.raises(ca.ALSError):
        lg.run_iter = -1
    lg.run_iter, lg.als_iter = 3, 5
    assert (lg.run_iter, lg.als_iter) == (3, 5)
    # a short buffer is refused and reports the size needed
    import ctypes as C

    n = C.c_size_t(4)
    buf = C.create_string_buffer(4)
    assert ca.lib().als_log_contents(lg._lg, buf, C.byref(n)) == ca.Status.INVALID_ARG
    assert n.value == len(lg.text().encode()) + 1
    # finishing an event that was never started: event_elapsed = now - 0, as the reference
    lg.event_finished(ca.EVENT_TYPE.ALS_UPDATE_V)
    last = E.parse(lg.text())[-1]
    assert last["text"] == "event ALS_UPDATE_V finished" and float(last["event_elapsed"]) > 1e9
    lg.close()


def test_ini_get(tmp_path):
    p = tmp_path / "x.ini"
    p.write_text("[general]\nlog_folder = log/toy_data ; where\nals_runs = 2\n[data]\nm = 15\n")
    assert ca.ini_get(str(p), "general", "log_folder") == "log/toy_data"
    assert ca.ini_get(str(p), "GENERAL", "als_runs") == "2"
    assert ca.ini_get(str(p), "general", "missing") == ""
    with pytest.raises(ca.ALSError) as e:
        ca.ini_get(str(tmp_path / "none.ini"), "general", "log_folder")
    assert e.value.status == ca.Status.IO


@pytest.fixture(scope="module")
def cpp_logger_exe(tmp_path_factory):
    """The reference-side script driver compiled against include/als_logger.hpp (through
    tests/cpp/logger.h) instead of the reference's logger.cpp."""
    out = tmp_path_factory.mktemp("cpplog") / "logger_driver"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", f"-I{ROOT / 'tests' / 'cpp'}",
           f"-I{ROOT / 'include'}", str(ROOT / "oracle" / "ref_logger_driver.cpp"), "-o",
           str(out), f"-L{LIBDIR}", "-lals_gb300", f"-Wl,-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_cpp_face_writes_what_the_reference_logger_writes(cpp_logger_exe, tmp_path):
    out = tmp_path / "log.csv"
    r = subprocess.run([str(cpp_logger_exe), str(out)], input=SCRIPT, capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    parsed = E.parse(out.read_text())
    assert E.check_columns(parsed) is None
    assert E.rows_of(parsed) == E.rows_of(E.parse((GOLDEN / "ref_log_script.csv").read_text()))
    assert E.echo_rows(r.stdout) == E.echo_rows((GOLDEN / "ref_log_script.stdout").read_text())


def test_live_against_the_reference_logger(tmp_path):
    """Where the reference's sources are present: a second script (one run, model saved, no
    per-iteration RMSE) through the reference's logger and through the library."""
    exe = ob.build_ref()
    if exe is None or not exe.exists():
        pytest.skip("the reference's logger.cpp is not present on this machine")
    params = E.params_text(32, 24, 20, 500, 50, 0.048, 2, "d", 1, "", 5, 3)
    calls = E.main_calls(params, als_runs=1, iters=2, iter_rmse=False, save_model=True,
                         final_rmse=[0.5])
    script = E.to_script(calls, write_cout=False, sleep_us=100)
    r = subprocess.run([str(exe), str(tmp_path / "ref.csv")], input=script, capture_output=True,
                       text=True, check=True)
    ref = E.parse((tmp_path / "ref.csv").read_text())
    lg = ca.logger()
    _replay(lg, script)
    ours = E.parse(lg.text())
    assert E.check_columns(ref) is None and E.check_columns(ours) is None
    assert E.rows_of(ours) == E.rows_of(ref) == E.expected_rows(calls)
    assert r.stdout == ""
    lg.close()


# ---------------------------------------------------------------------------------------------
# als_train with a log attached (GPU)


def _toy_model(toy, f, solve, iters):
    tr = ca.host_sparse_matrix(toy["m"], toy["n"], len(toy["R_train_csr_data"]))
    tr.set_csr(toy["R_train_csr_indptr"], toy["R_train_csr_indices"], toy["R_train_csr_data"])
    te = ca.host_sparse_matrix(toy["m"], toy["n"], len(toy["R_test_coo_data"]))
    te.set_coo(toy["R_test_coo_row"], toy["R_test_coo_col"], toy["R_test_coo_data"])
    return ca.als_model(tr, te, f, 0.05, iters, ca.CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR, solve)


def _oracle_rmse_per_iter(toy, f, iters, solve):
    m, n = toy["m"], toy["n"]
    csr = (toy["R_train_csr_indptr"], toy["R_train_csr_indices"], toy["R_train_csr_data"])
    csc = (toy["R_train_csc_indptr"], toy["R_train_csc_indices"], toy["R_train_csc_data"])
    test = (toy["R_test_coo_row"], toy["R_test_coo_col"], toy["R_test_coo_data"])
    out = []
    for k in range(1, iters + 1):
        U, V, _ = O.train(m, n, f, 0.05, k, csr, csc, solve=solve)
        out.append(O.rmse(*test, U, V))
    return out


def _split_rmse(rows):
    """Rows with the number of every "RMSE test: x" text replaced by "{rmse}", and the numbers."""
    vals, out = [], []
    for (i, r, a, ev, t) in rows:
        if t.startswith("RMSE test: "):
            vals.append(float(t.split(": ")[1]))
            t = "RMSE test: {rmse}"
        out.append((i, r, a, ev, t))
    return out, vals


@pytest.mark.gpu
@pytest.mark.parametrize("solve", [ca.SOLVE_TYPE.LU, ca.SOLVE_TYPE.CHOLESKY])
def test_train_writes_the_reference_training_lines(toy, solve, capfd):
    f, iters = (100 if toy["m"] == 15 else 20), 4
    with _toy_model(toy, f, solve, iters) as mdl:
        mdl.train()
        U0, V0 = mdl.h_UT.copy(), mdl.h_VT.copy()
        lg = ca.logger()
        lg.run_iter = 1
        mdl.set_logger(lg, iter_rmse=True, write_cout=True)
        mdl.train()
        assert (lg.run_iter, lg.als_iter) == (1, 0)
        # logging runs the epochs eagerly, half-sweep by half-sweep: same factors as the graph
        assert np.array_equal(mdl.h_UT, U0) and np.array_equal(mdl.h_VT, V0)
        mdl.set_logger(None)
    parsed = E.parse(lg.text())
    assert E.check_columns(parsed) is None
    got, vals = _split_rmse(E.rows_of(parsed))
    calls = E.train_calls(iters, True)
    exp = E.expected_rows([("run_iter", 1)] + calls)
    assert got == exp
    ref = _oracle_rmse_per_iter(toy, f, iters - 1, O.LU if solve == ca.SOLVE_TYPE.LU else O.CHOLESKY)
    assert np.allclose(vals, ref, atol=2e-4), (vals, ref)
    ev = [d for d in parsed if d["event_elapsed"]]
    assert all(float(d["event_elapsed"]) > 0 for d in ev)
    echo, _ = _split_rmse([(0,) + x for x in E.echo_rows(capfd.readouterr().out)])
    assert [x[1:] for x in echo] == [x[1:] for x in exp[1:]]
    lg.close()


@pytest.mark.gpu
def test_iterate_with_a_log_keeps_results_and_counts(toy):
    f = 100 if toy["m"] == 15 else 20
    with _toy_model(toy, f, ca.SOLVE_TYPE.CUMF_ALS_CG_FP32, 3) as mdl:
        mdl.init_factors()
        mdl.iterate(3)
        U0, V0 = mdl.get_factors()
        launches = mdl.counters()["launches"]
        lg = ca.logger()
        mdl.set_logger(lg)
        mdl.init_factors()
        mdl.iterate(3)
        U1, V1 = mdl.get_factors()
        assert np.array_equal(U0, U1) and np.array_equal(V0, V1)
        assert mdl.counters()["launches"] == launches  # launches of one epoch, both ways
        mdl.set_logger(None)
    rows = E.rows_of(E.parse(lg.text()))
    texts = [t for (_, _, _, _, t) in rows]
    assert texts.count("event ALS_ITER finished") == 3
    assert [a for (_, _, a, ev, t) in rows if t == "event ALS_UPDATE_U finished"] == [1, 2, 3]
    lg.close()
