"""Triples -> CSR / CSC (the reference's offline scipy step), the oracle side, on the CPU.

The restatement (oracle/coo.py) is pinned to the arrays the reference's toy prep scripts logged
(tests/golden/toy_data*.npz: the split's raw triples in, R_train_csr / R_train_csc /
R_test_coo out) and to scipy on random triples with duplicate cells."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_toy
from oracle import coo as OC


@pytest.mark.parametrize("name", ["toy_data", "toy_data_2"])
def test_oracle_builder_reproduces_the_reference_logs(name):
    d = load_toy(name)
    m, n = d["m"], d["n"]
    (ptr, idx, val), crow, (cptr, ridx, cval) = OC.coo_to_csr(
        m, n, d["raw_train_row"], d["raw_train_col"], d["raw_train_val"])
    assert np.array_equal(ptr, d["R_train_csr_indptr"])
    assert np.array_equal(idx, d["R_train_csr_indices"])
    assert np.array_equal(val, d["R_train_csr_data"].astype(np.float32))
    assert np.array_equal(cptr, d["R_train_csc_indptr"])
    assert np.array_equal(ridx, d["R_train_csc_indices"])
    assert np.array_equal(cval, d["R_train_csc_data"].astype(np.float32))
    # the test COO: coo_matrix(...).tocsr().tocoo() of the test triples
    tm = int(d["raw_test_row"].max()) + 1
    tn = int(d["raw_test_col"].max()) + 1
    (_, tidx, tval), trow, _ = OC.coo_to_csr(tm, tn, d["raw_test_row"], d["raw_test_col"],
                                             d["raw_test_val"])
    assert np.array_equal(trow, d["R_test_coo_row"])
    assert np.array_equal(tidx, d["R_test_coo_col"])
    assert np.array_equal(tval, d["R_test_coo_data"].astype(np.float32))


def random_triples(seed, rows, cols, n, dup_rate=0.3):
    rng = np.random.default_rng(seed)
    r = rng.integers(0, rows, n)
    c = rng.integers(0, cols, n)
    k = int(n * dup_rate)
    if k:  # repeat some cells, in scattered positions
        src = rng.integers(0, n, k)
        dst = rng.integers(0, n, k)
        r[dst], c[dst] = r[src], c[src]
    v = (rng.integers(1, 11, n) / 2).astype(np.float32)  # half stars
    return r.astype(np.int32), c.astype(np.int32), v


@pytest.mark.parametrize("seed,rows,cols,n", [(0, 300, 200, 20000), (1, 1, 1, 50), (2, 5, 7000, 300),
                                              (3, 9000, 3, 400), (4, 10, 10, 0)])
def test_oracle_builder_equals_scipy(seed, rows, cols, n):
    sp = pytest.importorskip("scipy.sparse")
    r, c, v = random_triples(seed, rows, cols, n)
    (ptr, idx, val), crow, (cptr, ridx, cval) = OC.coo_to_csr(rows, cols, r, c, v)
    A = sp.coo_matrix((v.astype(np.float64), (r, c)), shape=(rows, cols)).tocsr()
    assert np.array_equal(ptr, A.indptr) and np.array_equal(idx, A.indices)
    assert np.array_equal(val, A.data.astype(np.float32))
    assert np.array_equal(crow, A.tocoo().row)
    B = A.tocsc()
    assert np.array_equal(cptr, B.indptr) and np.array_equal(ridx, B.indices)
    assert np.array_equal(cval, B.data.astype(np.float32))
