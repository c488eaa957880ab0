"""The oracle-side build of the workload generator makes the library's bytes (CPU)."""
from __future__ import annotations

import numpy as np
import pytest

import cuda_als_gb300 as ca
from oracle import synth


@pytest.mark.parametrize("config,scale", [(1, 1.0), (2, 0.05), (3, 0.02), (4, 0.02), (5, 0.05)])
def test_oracle_generator_matches_the_library(config, scale):
    (ptr, idx, val), (tr_, tc, tv), info = synth.generate(config, scale=scale)
    tr, te, linfo = ca.synth_generate(config, scale=scale)
    assert info == {k: linfo[k] for k in info}
    assert np.array_equal(ptr, tr.h_csr_row_ptrs)
    assert np.array_equal(idx, tr.h_csr_coo_col_idxs)
    assert np.array_equal(val.view(np.uint32), tr.h_csr_coo_vals.view(np.uint32))
    assert np.array_equal(tr_, te.h_coo_row_idxs)
    assert np.array_equal(tc, te.h_csr_coo_col_idxs)
    assert np.array_equal(tv.view(np.uint32), te.h_csr_coo_vals.view(np.uint32))
