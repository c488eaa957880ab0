"""Regenerate tests/golden/ref_log_script.{txt,csv,stdout} with the reference's own logger.

oracle/build.py compiles the reference's logger.cpp (with oracle/ref_logger_driver.cpp, a
call-script driver) into oracle/_ref/.  This script feeds it the logger calls that the
reference's main.cpp + als_model::train make for two runs of three iterations with per-iteration
test RMSE lines (oracle.eventlog.main_calls, fixed RMSE texts), with a short sleep before every
call so the timestamp columns differ, and keeps the script, the CSV it saved and its stdout echo.
The tests check the oracle's restatement (line order, ids, counters, column relations, echo
format) and the library's log against these files on machines without the reference.

Run in a container that has the reference checked out:
    python tests/golden/make_log_fixture.py
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from oracle import build as ob  # noqa: E402
from oracle import eventlog as E  # noqa: E402

PARAMS = E.params_text(15, 13, 100, 143, 10, 0.05, 3, "data/toy_data", 2, "log/toy_data", 1, 2)
RMSE = [[1.25, 1.125], [1.25, 1.125]]
FINAL = [1.0625, 1.0625]


def script_calls():
    return E.main_calls(PARAMS, als_runs=2, iters=3, iter_rmse=True, save_model=False,
                        rmse=RMSE, final_rmse=FINAL)


def main():
    exe = ob.build_ref(verbose=True)
    if exe is None:
        sys.exit("the reference's logger.cpp is not present here")
    script = E.to_script(script_calls(), write_cout=True, sleep_us=300)
    with tempfile.TemporaryDirectory() as d:
        out = Path(d) / "log.csv"
        r = subprocess.run([str(exe), str(out)], input=script, capture_output=True, text=True,
                           check=True)
        (HERE / "ref_log_script.txt").write_text(script)
        (HERE / "ref_log_script.csv").write_text(out.read_text())
        (HERE / "ref_log_script.stdout").write_text(r.stdout)
    print("wrote", HERE / "ref_log_script.csv")


if __name__ == "__main__":
    main()
