"""CPU restatement of the reference's offline triples -> CSR / CSC step.  TEST INFRASTRUCTURE.

The reference's prep scripts turn a split's 1-based (user, item, rating) triples into
coo_matrix((r, (u - 1, i - 1))).tocsr().tocoo() (row-major entries, duplicates summed), .tocsr()
and .tocsc(), cast to float32 when written (data/toy_data/prepare_toy_data.py:108-110, 147-150,
201-208; data/netflix/prepare_netflix_data.py:88-109).  Restated with numpy: a stable sort by
(row, column), one entry per cell with its values summed in float64 in input order, one rounding
to float32; the CSC as the stable transpose (rows ascending within a column).
"""
from __future__ import annotations

import numpy as np


def coo_to_csr(rows: int, cols: int, r, c, v):
    """-> ((ptr, idx, val), coo_rows, (cptr, ridx, cval)), all int32 / float32."""
    r = np.asarray(r, np.int64)
    c = np.asarray(c, np.int64)
    v = np.asarray(v, np.float64)
    order = np.lexsort((c, r))  # stable: by row, then column, ties in input order
    rs, cs, vs = r[order], c[order], v[order]
    head = np.ones(len(rs), bool)
    head[1:] = (rs[1:] != rs[:-1]) | (cs[1:] != cs[:-1])
    starts = np.nonzero(head)[0]
    sums = np.add.reduceat(vs, starts) if len(vs) else np.zeros(0)
    # np.add.reduceat sums each cell left to right in float64: input order within the cell
    crow = rs[starts].astype(np.int32)
    idx = cs[starts].astype(np.int32)
    val = sums.astype(np.float32)
    ptr = np.zeros(rows + 1, np.int64)
    np.add.at(ptr, crow.astype(np.int64) + 1, 1)
    ptr = np.cumsum(ptr).astype(np.int32)
    t = np.argsort(idx, kind="stable")
    cptr = np.zeros(cols + 1, np.int64)
    np.add.at(cptr, idx.astype(np.int64) + 1, 1)
    return (ptr, idx, val), crow, (np.cumsum(cptr).astype(np.int32), crow[t], val[t])
