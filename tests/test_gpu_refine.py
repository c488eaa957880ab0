"""The FP64-residual refinement branch of the tensor-core Cholesky solve, driven on purpose.

After the FP32 Cholesky solve, one refinement step computes r = b - A x against the accumulator
copy of A.  On rows whose condition estimate (max L_jj / min L_jj)^2 exceeds `cond_threshold`
the residual's products and sums run in FP64; on the others in FP32.  An FP32 residual cannot
improve the forward error past cond(A) x 2^-24; an FP64 residual takes it to about
(cond(A) x 2^-24)^2.

The problem is built so the FP64 oracle's solution is the exact one: factor values k/8 and
integer ratings make every Gram entry and right-hand side exact in BF16 products and FP32 sums,
degrees are multiples of 8 and lambda = 2^-16, so lambda n_u and the regularised diagonal are
exact in FP32 too.  Column pairs that agree on all but 1% of the factor rows make each Gram
ill-conditioned (cond about 10^5.7, the Cholesky-diagonal estimate about 10^3.4).
"""
from __future__ import annotations

import numpy as np
import pytest

import cuda_als_gb300 as ca
from oracle import oracle as O

pytestmark = pytest.mark.gpu

F = 100
LAM = 2.0 ** -16


def _problem(seed=5):
    rng = np.random.default_rng(seed)
    m, n = 160, 3000
    Y = rng.integers(0, 7, (n, F)) / 8.0
    for j in range(0, 20, 2):  # near-collinear column pairs
        Y[:, j + 1] = Y[:, j]
        d = rng.random(n) < 0.01
        Y[d, j + 1] = np.clip(Y[d, j] + rng.choice([-1, 1], d.sum()) / 8.0, 0, 6 / 8.0)
    Y = Y.astype(np.float32)
    deg = 8 * rng.integers(40, 150, m)
    ptr = np.zeros(m + 1, np.int32)
    ptr[1:] = np.cumsum(deg)
    idx = np.concatenate([np.sort(rng.choice(n, d, replace=False)) for d in deg]).astype(np.int32)
    val = rng.integers(1, 6, len(idx)).astype(np.float32)
    return m, n, ptr, idx, val, Y


def _solve(m, n, ptr, idx, val, Y, refine_steps, cond_threshold):
    tr = ca.host_sparse_matrix(m, n, len(idx)).set_csr(ptr, idx, val)
    with ca.als_model(tr, None, F, LAM, 1, ca.CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR_TENSOR,
                      ca.SOLVE_TYPE.CHOLESKY, precision=int(ca.PRECISION.BF16),
                      refine_steps=refine_steps, cond_threshold=cond_threshold) as mdl:
        mdl.set_factors(np.zeros((m, F), np.float32), Y)
        mdl.half_sweep(0)
        U, _ = mdl.get_factors()
        c = mdl.counters()
    return U, c


def _row_err(U, Ue):
    d = np.linalg.norm(np.asarray(U, np.float64) - Ue, axis=1)
    return d / np.linalg.norm(Ue, axis=1)


def test_fp64_residual_refinement_runs_and_beats_fp32_refinement():
    m, n, ptr, idx, val, Y = _problem()
    Ue = np.zeros((m, F), np.float32)
    O.half_sweep(ptr, idx, val, Y, Ue, F, LAM, solve=O.CHOLESKY)  # FP64 (inputs exact in BF16)
    Ue = Ue.astype(np.float64)
    U64, c64 = _solve(m, n, ptr, idx, val, Y, 1, 1.0)      # every row takes the FP64 residual
    U32, c32 = _solve(m, n, ptr, idx, val, Y, 1, 1e30)     # none does
    U0, c0 = _solve(m, n, ptr, idx, val, Y, 0, 1.0)        # no refinement step at all
    assert c64["fp64_refined_rows"] == m
    assert c32["fp64_refined_rows"] == 0
    assert c0["fp64_refined_rows"] == 0  # nothing is refined without a refinement step
    for c in (c64, c32, c0):
        assert c["flagged_rows"] == 0
    e64, e32, e0 = _row_err(U64, Ue), _row_err(U32, Ue), _row_err(U0, Ue)
    # the FP64 residual lands near FP32 rounding of x; an FP32 residual stays at cond x 2^-24
    assert e64.max() < 1e-5, e64.max()
    assert np.median(e32) > 10 * e64.max(), (np.median(e32), e64.max())
    assert np.median(e0) > 10 * e64.max(), (np.median(e0), e64.max())
    # every row is closer to the FP64 solution with the FP64 residual than with the FP32 one
    assert (e64 < e32).all()
