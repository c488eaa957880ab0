"""Row-sharded ALS (cuda_als_gb300/sharded.py): the rating-balanced partition, and the half-sweep
split over ranks with an all-gather of the factor blocks and an all-reduced test RMSE.

CPU: world sizes 2 and 3 over gloo with the FP64 oracle solving each rank's block must reproduce
the single-process oracle training bit for bit (rows are independent; only where they are solved
changes).  GPU: two ranks on one GPU (gloo on the host, each rank its own handles; no kernel of one
rank waits on the other) must reproduce one handle's training bit for bit.
"""
from __future__ import annotations

import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

import _sharded_workers as W
import cuda_als_gb300 as ca
from oracle import oracle as O


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("nparts", [1, 2, 3, 5, 8])
@pytest.mark.parametrize("row_weight", [0.0, 10.0])
def test_partition_rows_covers_and_balances(nparts, row_weight):
    rng = np.random.default_rng(nparts)
    deg = np.minimum(rng.zipf(1.4, 500), 400)
    deg[[3, 70, 71]] = 0
    ptr = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
    b = ca.partition_rows(ptr, nparts, row_weight)
    assert b[0] == 0 and b[-1] == 500 and np.all(np.diff(b) >= 0)
    w = deg.astype(np.float64) + row_weight
    prefix = np.concatenate([[0.0], np.cumsum(w)])
    for k in range(1, nparts):   # every boundary within half a row's weight of its target
        assert abs(prefix[b[k]] - prefix[-1] * k / nparts) <= 0.5 * w.max() + 1e-9


def test_partition_rows_rejects_bad_arguments():
    ptr = np.array([0, 2, 1], np.int32)   # not monotone
    with pytest.raises(ca.ALSError):
        ca.partition_rows(ptr, 2)
    with pytest.raises(ca.ALSError):
        ca.partition_rows(np.array([0, 1], np.int32), 0)


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_oracle_reproduces_single_process(world, tmp_path):
    iters = 3
    mp.spawn(W.oracle_rank, args=(world, _free_port(), iters, str(tmp_path)), nprocs=world,
             join=True)
    z = np.load(tmp_path / "sharded.npz")
    tr, te, info = ca.synth_generate(1)
    m, n, f, lam = info["m"], info["n"], info["f"], info["lambda"]
    csr = (tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals)
    csc = O.csr_to_csc(m, n, *csr)
    U, V, _ = O.train(m, n, f, lam, iters, csr, csc, solve=O.CHOLESKY)
    assert np.array_equal(z["U"], U) and np.array_equal(z["V"], V)
    assert len(set(np.diff(z["ub"]))) > 0 and z["ub"][-1] == m and z["vb"][-1] == n
    rmse = O.rmse(te.h_coo_row_idxs, te.h_csr_coo_col_idxs, te.h_csr_coo_vals, U, V)
    assert float(z["rmse"]) == pytest.approx(rmse, rel=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,solve", [
    (ca.PRECISION.BF16, ca.SOLVE_TYPE.CHOLESKY),
    (ca.PRECISION.FP32, ca.SOLVE_TYPE.CUMF_ALS_CG_FP32),
])
def test_sharded_library_reproduces_one_handle(precision, solve, tmp_path):
    iters = 3
    tr, te, info = ca.synth_generate(2, scale=0.1)
    m, n, f, lam = info["m"], info["n"], info["f"], info["lambda"]
    _, V0 = O.init_factors(m, n, f)
    np.save(tmp_path / "V0.npy", V0)
    mp.spawn(W.library_rank, args=(2, _free_port(), iters, int(precision), int(solve),
                                   str(tmp_path)), nprocs=2, join=True)
    z = np.load(tmp_path / "sharded.npz")
    with ca.als_model(tr, te, f, lam, 1, ca.CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR_TENSOR, solve,
                      precision=int(precision)) as mdl:
        mdl.set_factors(np.zeros((m, f), np.float32), V0)
        mdl.iterate(iters)
        U, V = mdl.get_factors()
        rmse = mdl.rsme_test()
    assert np.array_equal(z["U"], U) and np.array_equal(z["V"], V)
    assert float(z["rmse"]) == pytest.approx(rmse, rel=1e-9)
