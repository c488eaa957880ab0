"""Regenerate tests/golden/toy_data*.npz from the reference's toy prep logs.

The reference's prep scripts (data/toy_data/prepare_toy_data.py,
data/toy_data_2/prepare_toy_data_2.py) print every array they write to disk, and their logs
(data/toy_data/prepare_toy_data.log, data/toy_data_2/prepare_toy_data_2.log) are committed in the
reference.  Those printed arrays are the only known-answer vectors the reference has: the train
CSR, the train CSC (scipy tocsc, i.e. the transpose) and the row-major test COO.  This script
parses them from the log text and stores them as small .npz fixtures.

It also re-derives the same arrays from the shipped ratings.dat with the scripts' own steps
(sklearn train_test_split(random_state=42), coo_matrix(...).tocsr().tocoo(), tocsr(), tocsc())
and asserts both agree, which pins the fixture to the reference's procedure as well as its log.

The re-derivation also stores the raw training and test triples of the split (0-based, in the
order train_test_split returns them, before any scipy conversion): the input of the GPU
triples -> CSR / CSC builder, whose output must equal the logged arrays.

Run in a container that has the reference checked out (the path as the first argument, or in
$CUDA_ALS_REFERENCE):
    python tests/golden/make_toy_fixtures.py /path/to/reference
"""
from __future__ import annotations

import os
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

TOYS = {
    # name: (log, ratings, m, n, test_size)
    "toy_data": ("data/toy_data/prepare_toy_data.log", "data/toy_data/ratings.dat", 15, 13, 10),
    "toy_data_2": ("data/toy_data_2/prepare_toy_data_2.log", "data/toy_data_2/ratings.dat", 32,
                   23, 20),
}

KEYS = ["R_test_coo.data", "R_test_coo.row", "R_test_coo.col", "R_train_csr.data",
        "R_train_csr.indptr", "R_train_csr.indices", "R_train_csc.data", "R_train_csc.indptr",
        "R_train_csc.indices"]


def parse_log(text: str) -> dict[str, np.ndarray]:
    """Each array is printed as a label line followed by numpy's bracketed repr."""
    out = {}
    for key in KEYS:
        m = re.search(r"^" + re.escape(key) + r"\s*\n\[([^\]]*)\]", text, re.M)
        if not m:
            raise ValueError(f"{key} not found in log")
        out[key] = np.array([int(tok) for tok in m.group(1).split()], dtype=np.int64)
    return out


def rederive(ratings: Path, m: int, n: int, test_size: int) -> dict[str, np.ndarray]:
    from scipy.sparse import coo_matrix
    from sklearn.model_selection import train_test_split

    rows = [line.split("::") for line in ratings.read_text().split() if line.strip()]
    user, item, rating = (np.array([int(r[i]) for r in rows], dtype=np.int32) for i in range(3))
    ui = np.vstack((user, item))
    ui_tr, ui_te, r_tr, r_te = train_test_split(ui.T, rating, test_size=test_size,
                                                random_state=42)
    te = coo_matrix((r_te, (ui_te[:, 0] - 1, ui_te[:, 1] - 1))).tocsr().tocoo()
    tr = coo_matrix((r_tr, (ui_tr[:, 0] - 1, ui_tr[:, 1] - 1)), shape=(m, n)).tocsr().tocoo()
    csr, csc = tr.tocsr(), tr.tocsc()
    raw = {"raw_train_row": ui_tr[:, 0] - 1, "raw_train_col": ui_tr[:, 1] - 1,
           "raw_train_val": r_tr, "raw_test_row": ui_te[:, 0] - 1,
           "raw_test_col": ui_te[:, 1] - 1, "raw_test_val": r_te}
    return {**raw, "R_test_coo.data": te.data, "R_test_coo.row": te.row, "R_test_coo.col": te.col,
            "R_train_csr.data": csr.data, "R_train_csr.indptr": csr.indptr,
            "R_train_csr.indices": csr.indices, "R_train_csc.data": csc.data,
            "R_train_csc.indptr": csc.indptr, "R_train_csc.indices": csc.indices}


def main(ref: Path) -> None:
    for name, (log, ratings, m, n, test_size) in TOYS.items():
        arrs = parse_log((ref / log).read_text())
        again = rederive(ref / ratings, m, n, test_size)  # needs sklearn and scipy
        for k in KEYS:
            assert np.array_equal(arrs[k], np.asarray(again[k], np.int64)), (name, k)
        print(f"{name}: log arrays == re-derived arrays")
        raw = {k: np.asarray(v, np.int64) for k, v in again.items() if k.startswith("raw_")}
        np.savez(HERE / f"{name}.npz", m=m, n=n,
                 **{k.replace(".", "_"): v for k, v in arrs.items()}, **raw)
        print(f"wrote {HERE / (name + '.npz')}")


if __name__ == "__main__":
    where = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CUDA_ALS_REFERENCE")
    if not where:
        sys.exit("usage: make_toy_fixtures.py REFERENCE_TREE (or set CUDA_ALS_REFERENCE)")
    main(Path(where))
