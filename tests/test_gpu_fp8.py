"""FP8 (e4m3) Gram and right-hand side on tcgen05 (kind::f8f6f4, FP32 accumulate in TMEM),
through the C ABI.

The FP8 sweep rounds the gathered factor table to e4m3 with one power-of-two scale per feature
(oracle/quant.py restates it) and the ratings to e4m3 (exact for star ratings).  e4m3 x e4m3
products are exact in FP32, so with the oracle run on the same rounded table the GPU must agree to
FP32-accumulation accuracy: a layout, descriptor or scaling mistake is an O(1) error.  Against the
unrounded FP64 solution the FP8 error budget is stated and measured separately.
"""
from __future__ import annotations

import numpy as np
import pytest

import cuda_als_gb300 as ca
from oracle import oracle as O
from oracle import quant
from test_gpu_tc import TOL_BF16_INPUTS, make_model, rel_rows, stage_boundary_problem

pytestmark = pytest.mark.gpu

FP8 = int(ca.PRECISION.FP8)


@pytest.mark.parametrize("f", [1, 10, 16, 31, 64, 100, 127, 128])
def test_fp8_half_sweep_matches_oracle_on_e4m3_inputs(f):
    rng, m, n, ptr, idx, val = stage_boundary_problem(f, seed=21)
    lam = 0.05
    U0 = (rng.standard_normal((m, f)) * 0.1).astype(np.float32)
    V0 = (rng.standard_normal((n, f)) * 0.3).astype(np.float32)
    with make_model(m, n, ptr, idx, val, f, lam, precision=FP8) as mdl:
        mdl.set_factors(U0, V0)
        mdl.half_sweep(0)
        U, _ = mdl.get_factors()
        assert mdl.counters()["flagged_rows"] == 0
        mdl.half_sweep(1)
        _, V = mdl.get_factors()
    Ue = U0.copy()
    O.half_sweep(ptr, idx, val, quant.e4m3_table(V0)[0], Ue, f, lam, solve=O.CHOLESKY)
    assert rel_rows(U, Ue) < TOL_BF16_INPUTS
    assert not U[np.diff(ptr) == 0].any()
    cptr, ridx, cval = O.csr_to_csc(m, n, ptr, idx, val)
    Ve = V0.copy()
    O.half_sweep(cptr, ridx, cval, quant.e4m3_table(U)[0], Ve, f, lam, solve=O.CHOLESKY)
    assert rel_rows(V, Ve) < TOL_BF16_INPUTS
    # against the unrounded FP64 solution: e4m3's 3 mantissa bits (2^-4 relative per factor)
    Uf = U0.copy()
    O.half_sweep(ptr, idx, val, V0, Uf, f, lam, solve=O.CHOLESKY)
    assert np.linalg.norm(U - Uf) / np.linalg.norm(Uf) < 0.15


@pytest.mark.parametrize("solve,f", [(ca.SOLVE_TYPE.LU, 100), (ca.SOLVE_TYPE.CUMF_ALS_CG_FP32, 100),
                                     (ca.SOLVE_TYPE.CUMF_ALS_CG_FP32, 128),
                                     (ca.SOLVE_TYPE.CUMF_ALS_CG_FP32, 64),
                                     (ca.SOLVE_TYPE.LU, 128)])
def test_fp8_other_solvers(solve, f):
    rng, m, n, ptr, idx, val = stage_boundary_problem(f, seed=27)
    U0 = (rng.standard_normal((m, f)) * 0.1).astype(np.float32)
    V0 = (rng.standard_normal((n, f)) * 0.3).astype(np.float32)
    with make_model(m, n, ptr, idx, val, f, solve=solve, cg_tol=0.0, precision=FP8) as mdl:
        mdl.set_factors(U0, V0)
        mdl.half_sweep(0)
        U, _ = mdl.get_factors()
    osolve = O.LU if solve == ca.SOLVE_TYPE.LU else O.CG_FP32
    Ue = U0.copy()
    O.half_sweep(ptr, idx, val, quant.e4m3_table(V0)[0], Ue, f, 0.05, solve=osolve, cg_tol=0.0)
    assert rel_rows(U, Ue) < (TOL_BF16_INPUTS if osolve == O.LU else 1e-3)


@pytest.mark.parametrize("f", [16, 64, 100, 112, 128])
def test_fp8_cg16_on_general_factors(f):
    """The FP16-Gram CG with its products on the tensor core, from an FP8 Gram.  Up to f = 112
    the ratings ride in the Gram's MMA as feature column ng (one MMA per 32 ratings); at f = 128
    there is no free column and the right-hand side takes its own N = 16 MMA."""
    rng, m, n, ptr, idx, val = stage_boundary_problem(f, seed=29)
    U0 = (rng.standard_normal((m, f)) * 0.1).astype(np.float32)
    V0 = (rng.standard_normal((n, f)) * 0.3).astype(np.float32)
    with make_model(m, n, ptr, idx, val, f, solve=ca.SOLVE_TYPE.CUMF_ALS_CG_FP16, cg_tol=0.0,
                    precision=FP8) as mdl:
        mdl.set_factors(U0, V0)
        mdl.half_sweep(0)
        U, _ = mdl.get_factors()
    Ue = U0.copy()
    O.half_sweep(ptr, idx, val, quant.e4m3_table(V0)[0], Ue, f, 0.05, solve=O.CG_FP16,
                 cg_tol=0.0)
    d = np.asarray(U, np.float64) - Ue
    assert np.linalg.norm(d) / np.linalg.norm(Ue) < 2e-3
    assert rel_rows(U, Ue) < 5e-2


def test_fp8_heavy_rows_many_stages():
    rng = np.random.default_rng(3)
    m, n, f = 64, 6000, 128
    degrees = rng.integers(1, 40, m)
    degrees[:4] = [5999, 4096, 3000, 2049]
    from conftest import random_csr
    ptr, idx, val = random_csr(rng, m, n, degrees=degrees)
    V0 = (rng.standard_normal((n, f)) * 0.2).astype(np.float32)
    with make_model(m, n, ptr, idx, val, f, precision=FP8) as mdl:
        mdl.set_factors(np.zeros((m, f), np.float32), V0)
        mdl.half_sweep(0)
        U, _ = mdl.get_factors()
    Ue = np.zeros((m, f), np.float32)
    O.half_sweep(ptr, idx, val, quant.e4m3_table(V0)[0], Ue, f, 0.05, solve=O.CHOLESKY)
    assert rel_rows(U, Ue) < TOL_BF16_INPUTS


def test_fp8_fused_rhs_on_heavy_rows():
    """Rows of up to 5,999 ratings (94 stages) through the tensor-core CG at f = 100, where the
    e4m3 ratings ride in the Gram's MMA as feature column 112."""
    rng = np.random.default_rng(5)
    m, n, f = 64, 6000, 100
    degrees = rng.integers(1, 40, m)
    degrees[:4] = [5999, 4096, 3000, 2049]
    from conftest import random_csr
    ptr, idx, val = random_csr(rng, m, n, degrees=degrees)
    V0 = (rng.standard_normal((n, f)) * 0.2).astype(np.float32)
    with make_model(m, n, ptr, idx, val, f, solve=ca.SOLVE_TYPE.CUMF_ALS_CG_FP16, cg_tol=0.0,
                    precision=FP8) as mdl:
        mdl.set_factors(np.zeros((m, f), np.float32), V0)
        mdl.half_sweep(0)
        U, _ = mdl.get_factors()
    Ue = np.zeros((m, f), np.float32)
    O.half_sweep(ptr, idx, val, quant.e4m3_table(V0)[0], Ue, f, 0.05, solve=O.CG_FP16,
                 cg_tol=0.0)
    d = np.asarray(U, np.float64) - Ue
    assert np.linalg.norm(d) / np.linalg.norm(Ue) < 2e-3


def test_fp8_training_on_the_transposed_netflix_shape():
    """Scaled workload 4 (f = 128), 10 iterations from the srand(0) init: FP8, BF16 and FP32
    test RMSE against the FP64 oracle's training.  Stated per precision: BF16 within 2e-3 of
    FP64, FP8 within 3e-2 (e4m3 keeps 3 mantissa bits of every factor)."""
    tr, te, info = ca.synth_generate(4, scale=0.1)
    m, n, f, lam = info["m"], info["n"], info["f"], info["lambda"]
    csr = (tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals)
    test = (te.h_coo_row_idxs, te.h_csr_coo_col_idxs, te.h_csr_coo_vals)
    csc = O.csr_to_csc(m, n, *csr)
    Ue, Ve, _ = O.train(m, n, f, lam, 10, csr, csc, solve=O.CHOLESKY)
    r64 = O.rmse(*test, Ue, Ve)
    out = {}
    for prec in (ca.PRECISION.FP32, ca.PRECISION.BF16, ca.PRECISION.FP8):
        with ca.als_model(tr, te, f, lam, 10, ca.CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR_TENSOR,
                          ca.SOLVE_TYPE.CHOLESKY, precision=int(prec)) as mdl:
            mdl.train()
            out[prec] = mdl.rsme_test()
            assert mdl.counters()["flagged_rows"] == 0
    print({p.name: (out[p], abs(out[p] - r64)) for p in out}, "fp64", r64)
    assert abs(out[ca.PRECISION.FP32] - r64) < 1e-4
    assert abs(out[ca.PRECISION.BF16] - r64) < 2e-3
    assert abs(out[ca.PRECISION.FP8] - r64) < 3e-2
