"""Row-sharded ALS over torch.distributed ranks.

Within a half-sweep every row is independent given the opposite factor table, so the rows of each
side split into contiguous, rating-balanced blocks (als_partition_rows), one per rank.  Every rank
keeps both full factor tables; a half-sweep solves the rank's block of rows against the full
opposite table and one all-gather of the updated blocks rebuilds the table on every rank (rows * f
floats in total).  The test RMSE is one FP64 all-reduce of the ranks' squared-error sums.

This replaces the reference's single-GPU loop over m_batches / n_batches row batches
(als_model.cu:1891-1896, main.cpp:46-47) when a half-sweep is spread over several GPUs.  The solve
of a block is delegated to a backend object:

    backend.solve(side, X_local, Y_full) -> X_local   # side 0: U rows of the block given V
                                                      # side 1: V rows of the block given U
    backend.sse(U_local, V_full) -> (sum of squared test errors, count) for the block's test rows

`LibraryBackend` runs both on the GPU through the C ABI (two handles per rank: the block's CSR rows
for U, and the block's CSC columns as the rows of the transposed problem for V).  Any object with
the same two methods works; the collective runs on whatever backend the process group uses (gloo
exchanges host tensors, nccl device tensors).
"""
from __future__ import annotations

import numpy as np

from . import CALCULATE_VTVS_TYPE, SOLVE_TYPE, als_model, host_sparse_matrix, partition_rows

__all__ = ["LibraryBackend", "sharded_als_model", "row_block"]


def row_block(ptr, idx, val, lo: int, hi: int):
    """Rows [lo, hi) of a CSR (or columns of a CSC) as a stand-alone CSR: (ptr, idx, val)."""
    ptr = np.asarray(ptr)
    b, e = int(ptr[lo]), int(ptr[hi])
    return ((ptr[lo:hi + 1] - b).astype(np.int32), np.ascontiguousarray(idx[b:e], np.int32),
            np.ascontiguousarray(val[b:e], np.float32))


class LibraryBackend:
    """A rank's two blocks solved by libals_gb300 handles (one per side)."""

    def __init__(self, block_u, block_v, m, n, f, lam, test=None,
                 vtvs=CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR_TENSOR, solve=SOLVE_TYPE.AUTO, **options):
        (pu, iu, vu), (pv, iv, vv) = block_u, block_v
        mu, nv = len(pu) - 1, len(pv) - 1
        self.f = f
        self.n_test = 0 if test is None else len(test[2])
        self.hu = self.hv = None  # a rank may own no rows of a side
        if mu > 0:
            tr_u = host_sparse_matrix(mu, n, len(iu)).set_csr(pu, iu, vu)
            te_u = None
            if self.n_test:
                te_u = host_sparse_matrix(mu, n, self.n_test).set_coo(*test)
            self.hu = als_model(tr_u, te_u, f, lam, 1, vtvs, solve, **options)
        if nv > 0:
            tr_v = host_sparse_matrix(nv, m, len(iv)).set_csr(pv, iv, vv)
            self.hv = als_model(tr_v, None, f, lam, 1, vtvs, solve, **options)

    def solve(self, side, X_local, Y_full):
        h = self.hu if side == 0 else self.hv
        if h is None:
            return np.zeros((0, self.f), np.float32)
        h.set_factors(np.ascontiguousarray(X_local, np.float32),
                      np.ascontiguousarray(Y_full, np.float32))
        h.half_sweep(0)
        return h.get_factors()[0]

    def sse(self, U_local, V_full):
        if self.n_test == 0 or self.hu is None:
            return 0.0, 0
        self.hu.set_factors(np.ascontiguousarray(U_local, np.float32),
                            np.ascontiguousarray(V_full, np.float32))
        r = self.hu.rsme_test()  # FP64 on the device
        return r * r * self.n_test, self.n_test

    def close(self):
        for h in (self.hu, self.hv):
            if h is not None:
                h.close()


class sharded_als_model:
    """ALS with the rows of each half-sweep spread over the ranks of a process group.

    csr / csc: (ptr, idx, val) of the whole training matrix (every rank passes the same arrays);
    V0: the initial item table (n x f; U starts at zero, as als_model.cu:1772-1777);
    make_backend(block_u, block_v, test_block) -> backend for this rank's blocks;
    test: optional (rows, cols, vals) of the held-out ratings;
    row_weight: the solve's cost per row in rating-equivalents for the partition.
    """

    def __init__(self, m, n, f, csr, csc, V0, make_backend, group=None, test=None,
                 row_weight=0.0, device="cpu"):
        import torch.distributed as dist

        self.dist, self.group, self.device = dist, group, device
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        self.m, self.n, self.f = m, n, f
        self.ub = partition_rows(csr[0], self.world, row_weight)
        self.vb = partition_rows(csc[0], self.world, row_weight)
        ulo, uhi = int(self.ub[self.rank]), int(self.ub[self.rank + 1])
        vlo, vhi = int(self.vb[self.rank]), int(self.vb[self.rank + 1])
        self.ulo, self.uhi, self.vlo, self.vhi = ulo, uhi, vlo, vhi
        block_u = row_block(*csr, ulo, uhi)
        block_v = row_block(*csc, vlo, vhi)
        test_block = None
        if test is not None:
            rows, cols, vals = (np.asarray(a) for a in test)
            sel = (rows >= ulo) & (rows < uhi)
            test_block = ((rows[sel] - ulo).astype(np.int32), cols[sel].astype(np.int32),
                          vals[sel].astype(np.float32))
        self.n_test = 0 if test is None else len(test[2])
        self.backend = make_backend(block_u, block_v, test_block)
        self.U = np.zeros((m, f), np.float32)
        self.V = np.ascontiguousarray(V0, np.float32).copy()

    def _gather(self, local, bounds):
        """All-gather of the ranks' row blocks (padded to the largest) into the full table."""
        import torch

        rows = int(np.max(np.diff(bounds)))
        buf = np.zeros((max(rows, 1), self.f), np.float32)
        buf[:len(local)] = local
        mine = torch.from_numpy(buf).to(self.device)
        parts = [torch.empty_like(mine) for _ in range(self.world)]
        self.dist.all_gather(parts, mine, group=self.group)
        out = np.empty((int(bounds[-1]), self.f), np.float32)
        for k, t in enumerate(parts):
            lo, hi = int(bounds[k]), int(bounds[k + 1])
            out[lo:hi] = t.cpu().numpy()[:hi - lo]
        return out

    def half_sweep(self, side: int):
        if side == 0:
            local = self.backend.solve(0, self.U[self.ulo:self.uhi], self.V)
            self.U = self._gather(local, self.ub)
        else:
            local = self.backend.solve(1, self.V[self.vlo:self.vhi], self.U)
            self.V = self._gather(local, self.vb)

    def iterate(self, iters: int):
        for _ in range(iters):
            self.half_sweep(0)
            self.half_sweep(1)

    def rsme_test(self) -> float:
        """sqrt(sum of squared test errors / count) over all ranks (one FP64 all-reduce)."""
        import torch

        sse, cnt = self.backend.sse(self.U[self.ulo:self.uhi], self.V)
        t = torch.tensor([float(sse), float(cnt)], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, group=self.group)
        return float(np.sqrt(t[0].item() / t[1].item())) if t[1].item() > 0 else 0.0

    def close(self):
        if hasattr(self.backend, "close"):
            self.backend.close()
