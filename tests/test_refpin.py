"""The oracle's floating point pinned to the reference's own CUDA path (CPU).

`tests/golden/refkernels_workload1.npz` holds outputs of the reference's half-sweep run on a GB300
by `tests/golden/make_refkernel_fixtures.py`: its `calculate_vtvs` Gram kernel
(als_model.cu:91-167) and `updateXWithCGKernel` (cumf_als_cg/cg.cu:37-232), built from its sources
into cubins, and cuBLAS batched LU without pivoting as `LU_solve_U` (als_model.cu:1570-1644) calls
it, on workload 1 from the srand(0) init.  The oracle must reproduce them:

* the Gram and the LU path to FP32 rounding (one half-sweep 1e-5, ten iterations 1e-4, RMSE 1e-5);
* the CG path at f = 32: one half-sweep to 2e-5 (FP32 and FP64 oracle).  Ten iterations of FP32
  CG drift apart in any two implementations (the unconverged 6-step solves and the r'r < 1e-4
  exit amplify summation-order differences: 9e-4 between the oracle's FP32 mode and the
  reference, about as far as the library's own FP32 path), so there the bar is 2e-3 on the
  factors and 1e-4 on the test RMSE.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import cuda_als_gb300 as ca
from oracle import oracle as O
from oracle import refkernels as RK

FIX = Path(__file__).with_name("golden") / "refkernels_workload1.npz"


@pytest.fixture(scope="module")
def ref():
    d = np.load(FIX)
    tr, te, info = ca.synth_generate(1)
    m, n, lam = info["m"], info["n"], info["lambda"]
    csr = (tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals)
    test = (te.h_coo_row_idxs, te.h_csr_coo_col_idxs, te.h_csr_coo_vals)
    return d, m, n, lam, csr, O.csr_to_csc(m, n, *csr), test


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_reference_gram_is_the_fp64_gram(ref):
    d, m, n, lam, csr, csc, test = ref
    f = 10
    _, V0 = O.init_factors(m, n, f)
    ptr, idx = csr[0], csr[1]
    for k, u in enumerate(d["gram_rows"]):
        Y = V0[idx[ptr[u]:ptr[u + 1]]].astype(np.float64)
        assert _rel(d["gram"][k], Y.T @ Y + lam * len(Y) * np.eye(f)) < 1e-6


def test_oracle_lu_reproduces_the_reference(ref):
    d, m, n, lam, csr, csc, test = ref
    f = 10
    U0, V0 = O.init_factors(m, n, f)
    X = U0.copy()
    O.half_sweep(*csr, V0, X, f, lam, solve=O.LU)
    assert _rel(X, d["lu_half_U"]) < 1e-5
    U, V, flagged = O.train(m, n, f, lam, 10, csr, csc, solve=O.LU)
    assert flagged == 0
    assert _rel(U, d["lu_U"]) < 1e-4
    assert _rel(V, d["lu_V"]) < 1e-4
    assert abs(O.rmse(*test, U, V) - float(d["lu_rmse"])) < 1e-5


def test_oracle_cg_reproduces_the_reference(ref):
    d, m, n, lam, csr, csc, test = ref
    f = 32
    U0, V0 = O.init_factors(m, n, f)
    for fp32 in (True, False):
        X = U0.copy()
        O.half_sweep(*csr, V0, X, f, lam, solve=O.CG_FP32, fp32=fp32)
        assert _rel(X, d["cg_half_U"]) < 2e-5
    U, V, _ = O.train(m, n, f, lam, 10, csr, csc, solve=O.CG_FP32, fp32=True)
    assert _rel(V, d["cg_V"]) < 2e-3
    assert abs(O.rmse(*test, U, V) - float(d["cg_rmse"])) < 1e-4


def test_reference_launches_stay_within_the_kernels_int_offsets():
    """The reference's kernels offset the Gram buffer by blockIdx.x * f * f in int: every launch of
    them (oracle/refkernels.py) covers at most batch_rows(f) rows, the most that stay below 2^31."""
    for f in (10, 32, 64, 100, 128):
        b = RK.batch_rows(f)
        assert (b - 1) * f * f + f * f - 1 < 2**31 <= (b + 1) * f * f
