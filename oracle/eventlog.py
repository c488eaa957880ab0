"""The reference's event log, restated: which lines its USE_LOGGER build writes and in which
order, and how the CSV columns relate.  TEST INFRASTRUCTURE ONLY.

Only tests/ import this module; it is the checker for the library's als_log_* calls, the
als_train hooks and the command-line driver, never part of them.

Pinned by tests/golden/ref_log_script.csv, the CSV the reference's own logger (logger.cpp,
compiled from its sources by oracle/build.py) wrote for the script of `main_calls` below
(tests/golden/make_log_fixture.py), and live against that build where the reference tree is
present.
"""
from __future__ import annotations

import csv
import io
import re

HEADER = ["log_name", "id", "run_iter", "als_iter", "prev_ts", "curr_ts", "elapsed",
          "event_elapsed", "text"]                                  # logger.cpp:71
EVENTS = ["ALS_UPDATE_U", "ALS_UPDATE_V", "ALS_ITER", "MF_MODEL_TRAINING"]  # logger.h:8-13
VTVS = ["SIMPLE", "SMEM_ROW_MAJOR", "SMEM_COL_MAJOR", "SMEM_ROW_MAJOR_NO_CALC",
        "SMEM_COL_MAJOR_TWO_THREADS", "SMEM_ROW_MAJOR_TENSOR", "SMEM_ROW_MAJOR_TENSOR_SYMMETRIC",
        "SMEM_ROW_MAJOR_TENSOR_SYMMETRIC_MULT_FRAG"]               # als_model.h:12-21
SOLVE = ["LU", "CUMF_ALS_CG_FP16", "CUMF_ALS_CG_FP32", "CHOLESKY", "AUTO"]
NAME_RE = re.compile(r"^\d{8}_\d{6}_debug=false\.csv$")          # logger.cpp:48-69

# Lines the reference's half-sweeps write between their stages (cuSPARSE/cuBLAS product, Gram
# kernel per batch, batched solver per batch: als_model.cu:1857-2014, :2092-2252).  The sweep
# here is one fused kernel per bucket, so it has no such boundaries and writes none of them.
STAGE_PREFIXES = ("VTRT via", "UTR via", "vtvs ", "utus ", "U solver done", "V solver done")


def train_calls(iters: int, iter_rmse: bool, rmse=None):
    """Logger calls of als_model::train (als_model.cu:1766-2289), stage lines left out.

    Calls: ("log", text) | ("start", event) | ("finish", event) | ("als_iter", k).
    rmse: per-iteration test RMSE values for the "RMSE test" lines (CALC_ITER_RMSE build,
    :2269-2274), or None to leave "{rmse}" in the text."""
    calls = [("log", "als model training started"),          # :1769
             ("log", "factors initialization done")]          # :1787
    for it in range(iters):
        calls += [("als_iter", it + 1), ("start", "ALS_ITER"),           # :1793-1794
                  ("start", "ALS_UPDATE_U"), ("finish", "ALS_UPDATE_U"),  # :1801, :2022
                  ("start", "ALS_UPDATE_V"), ("finish", "ALS_UPDATE_V"),  # :2034, :2260
                  ("finish", "ALS_ITER")]                                 # :2261
        if iter_rmse and it < iters - 1:
            v = "{rmse}" if rmse is None else "%f" % float(rmse[it])    # std::to_string(float)
            calls.append(("log", "RMSE test: " + v))
    calls += [("als_iter", 0), ("log", "als model training done")]       # :2278, :2287
    return calls


def params_text(m, n, f, nnz_train, nnz_test, lam, iters, data_folder, als_runs, log_folder,
                vtvs, solve, smem_col_cnt=32):
    """The parameter line of main.cpp:54-60 (a default-formatted stream: %g for lambda)."""
    return (f"m={m} n={n} f={f} nnz_train={nnz_train} nnz_test={nnz_test} "
            f"lambda={'%g' % float(lam)} als_iters={iters} data_folder={data_folder} "
            f"als_runs={als_runs} log_folder={log_folder} als_calculate_vtvs_type={VTVS[vtvs]} "
            f"als_solve_type={SOLVE[solve]} smem_col_cnt={smem_col_cnt}")


def main_calls(params: str, als_runs: int, iters: int, iter_rmse: bool, save_model: bool,
               rmse=None, final_rmse=None):
    """Logger calls of main.cpp:48-122 around train_calls (the lines after g_logger.init).

    rmse[r] / final_rmse[r]: the per-iteration / final test RMSE of run r, or None for
    "{rmse}" placeholders."""
    calls = [("log", params),                                               # :62
             ("log", "host train and test ratings loaded")]                 # :78
    for r in range(als_runs):
        calls += [("start", "MF_MODEL_TRAINING"), ("run_iter", r + 1),      # :86-88
                  ("log", "als model constructor done")]                    # :94
        calls += train_calls(iters, iter_rmse, None if rmse is None else rmse[r])
        fin = "{rmse}" if final_rmse is None else "%f" % float(final_rmse[r])
        calls += [("finish", "MF_MODEL_TRAINING"),                          # :101
                  ("log", "final RMSE test: " + fin)]                       # :105
        if als_runs == 1 and save_model:
            calls.append(("log", "saved model in cumf_sgd libmf format"))   # :110
    calls += [("run_iter", 0), ("log", "all als runs done")]                # :116-119
    return calls


def expected_rows(calls):
    """(id, run_iter, als_iter, is_event, text) of the lines a logger writes for `calls`,
    starting with init's "init logger" line (logger.cpp:72)."""
    rows = [(0, 0, 0, False, "init logger")]
    run_iter = als_iter = 0
    for c in calls:
        if c[0] == "run_iter":
            run_iter = c[1]
        elif c[0] == "als_iter":
            als_iter = c[1]
        elif c[0] == "log":
            rows.append((len(rows), run_iter, als_iter, False, c[1]))
        elif c[0] == "finish":
            rows.append((len(rows), run_iter, als_iter, True, f"event {c[1]} finished"))
    return rows


def to_script(calls, write_cout=True, sleep_us=0):
    """The call list as the ref_logger driver's stdin script (oracle/ref_logger_driver.cpp)."""
    out, run_iter, als_iter = [], 0, 0
    for c in calls:
        if c[0] in ("run_iter", "als_iter"):
            run_iter, als_iter = (c[1], als_iter) if c[0] == "run_iter" else (run_iter, c[1])
            out.append(f"iters {run_iter} {als_iter}")
            continue
        if sleep_us:
            out.append(f"sleep_us {sleep_us}")
        if c[0] == "log":
            out.append(f"log {int(write_cout)} {c[1]}")
        elif c[0] == "start":
            out.append(f"start {EVENTS.index(c[1])}")
        elif c[0] == "finish":
            out.append(f"finish {EVENTS.index(c[1])} {int(write_cout)}")
    return "\n".join(out) + "\n"


def parse(text: str):
    """CSV text -> list of dict rows (the header must be logger.cpp:71's)."""
    r = list(csv.reader(io.StringIO(text)))
    assert r and r[0] == HEADER, r[:1]
    return [dict(zip(HEADER, row)) for row in r[1:] if row]


def rows_of(parsed):
    return [(int(d["id"]), int(d["run_iter"]), int(d["als_iter"]), d["event_elapsed"] != "",
             d["text"]) for d in parsed]


def check_columns(parsed, tol=2.5e-6):
    """The column relations of logger.cpp:75-87 and :108-143 (timestamps printed with 6
    decimals, so differences of printed values agree to within 2 units of the last place):
    * one log_name of the form %Y%m%d_%H%M%S_debug=false.csv; ids 0, 1, 2, ...;
    * a text line advances prev_ts before printing it: prev_ts == curr_ts, and its elapsed is
      curr_ts minus the previous text line's curr_ts; event_elapsed is empty;
    * an event line prints the last text line's timestamp as prev_ts without advancing it:
      elapsed == curr_ts - prev_ts, event_elapsed a number >= 0;
    * curr_ts never decreases.
    Returns None when every relation holds, else a message naming the first line that breaks."""
    names = {d["log_name"] for d in parsed}
    if len(names) != 1 or not NAME_RE.match(next(iter(names))):
        return f"log_name {names}"
    last_text_ts = None
    prev_curr = -1.0
    for k, d in enumerate(parsed):
        if int(d["id"]) != k:
            return f"line {k}: id {d['id']}"
        prev_ts, curr = float(d["prev_ts"]), float(d["curr_ts"])
        elapsed = float(d["elapsed"])
        if curr < prev_curr:
            return f"line {k}: curr_ts decreases"
        prev_curr = curr
        if d["event_elapsed"] == "":
            if abs(prev_ts - curr) > tol:
                return f"line {k}: text line prev_ts != curr_ts"
            if last_text_ts is not None and abs(elapsed - (curr - last_text_ts)) > tol:
                return f"line {k}: text elapsed != curr_ts - previous text curr_ts"
            last_text_ts = curr
        else:
            if last_text_ts is not None and abs(prev_ts - last_text_ts) > tol:
                return f"line {k}: event prev_ts is not the last text line's time"
            if abs(elapsed - (curr - prev_ts)) > tol:
                return f"line {k}: event elapsed != curr_ts - prev_ts"
            if float(d["event_elapsed"]) < 0:
                return f"line {k}: negative event_elapsed"
            if not d["text"].startswith("event ") or not d["text"].endswith(" finished"):
                return f"line {k}: event text {d['text']!r}"
    return None


ECHO_RE = re.compile(r"^run iter: (\d+) als iter: (\d+) elapsed: (\d+\.\d{6})"
                     r"(?: event elapsed: (\d+\.\d{6}))? (.*)$")


def echo_rows(stdout: str):
    """(run_iter, als_iter, is_event, text) of the stdout echo lines (logger.cpp:84-86,
    :140-142; std::fixed as main.cpp:52)."""
    out = []
    for line in stdout.splitlines():
        mt = ECHO_RE.match(line)
        if mt:
            out.append((int(mt.group(1)), int(mt.group(2)), mt.group(4) is not None, mt.group(5)))
    return out
