"""Rank bodies for tests/test_sharded.py (spawned processes import this module)."""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


class OracleBackend:
    """The block solves by the FP64 oracle (test infrastructure): same rows, same arithmetic as a
    single-process oracle sweep, so the sharded result must match it bit for bit."""

    def __init__(self, block_u, block_v, test, f, lam):
        from oracle import oracle as O

        self.O, self.bu, self.bv, self.test, self.f, self.lam = O, block_u, block_v, test, f, lam

    def solve(self, side, X_local, Y_full):
        ptr, idx, val = self.bu if side == 0 else self.bv
        X = np.ascontiguousarray(X_local, np.float32).copy()
        if len(ptr) > 1:
            self.O.half_sweep(ptr, idx, val, Y_full, X, self.f, self.lam, solve=self.O.CHOLESKY)
        return X

    def sse(self, U_local, V_full):
        if self.test is None or len(self.test[2]) == 0:
            return 0.0, 0
        rows, cols, vals = self.test
        pred = np.einsum("ij,ij->i", U_local[rows].astype(np.float64), V_full[cols].astype(np.float64))
        return float(np.sum((vals.astype(np.float64) - pred) ** 2)), len(vals)


def _init(rank, world, port):
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    return dist


def oracle_rank(rank, world, port, iters, out_dir):
    import cuda_als_gb300 as ca
    from cuda_als_gb300.sharded import sharded_als_model
    from oracle import oracle as O

    dist = _init(rank, world, port)
    tr, te, info = ca.synth_generate(1)
    m, n, f, lam = info["m"], info["n"], info["f"], info["lambda"]
    csr = (tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals)
    csc = O.csr_to_csc(m, n, *csr)
    test = (te.h_coo_row_idxs, te.h_csr_coo_col_idxs, te.h_csr_coo_vals)
    _, V0 = O.init_factors(m, n, f)
    model = sharded_als_model(m, n, f, csr, csc, V0,
                              lambda bu, bv, tb: OracleBackend(bu, bv, tb, f, lam),
                              test=test, row_weight=float(f))
    model.iterate(iters)
    rmse = model.rsme_test()
    if rank == 0:
        np.savez(os.path.join(out_dir, "sharded.npz"), U=model.U, V=model.V, rmse=rmse,
                 ub=model.ub, vb=model.vb)
    dist.barrier()
    dist.destroy_process_group()


def library_rank(rank, world, port, iters, precision, solve, out_dir):
    import cuda_als_gb300 as ca
    from cuda_als_gb300.sharded import LibraryBackend, sharded_als_model

    dist = _init(rank, world, port)
    tr, te, info = ca.synth_generate(2, scale=0.1)
    m, n, f, lam = info["m"], info["n"], info["f"], info["lambda"]
    csr = (tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals)
    csc = ca.csr_to_csc(m, n, *csr)
    test = (te.h_coo_row_idxs, te.h_csr_coo_col_idxs, te.h_csr_coo_vals)
    V0 = np.load(os.path.join(out_dir, "V0.npy"))
    opts = dict(precision=int(precision))
    model = sharded_als_model(
        m, n, f, csr, csc, V0,
        lambda bu, bv, tb: LibraryBackend(bu, bv, m, n, f, lam, tb, solve=solve, **opts),
        test=test)
    model.iterate(iters)
    rmse = model.rsme_test()
    if rank == 0:
        np.savez(os.path.join(out_dir, "sharded.npz"), U=model.U, V=model.V, rmse=rmse)
    model.close()
    dist.barrier()
    dist.destroy_process_group()
