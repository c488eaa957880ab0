"""Tensor-core (tcgen05, BF16 operands, FP32 accumulate) half-sweep parity through the C ABI.

The tight check runs the FP64 oracle on the BF16-rounded opposite factors: BF16 x BF16 products
are exact in FP32 and the ratings are exact in BF16, so the tensor-core Gram and right-hand side
must then agree with FP64 to FP32-accumulation accuracy.  Any operand-layout, descriptor or
TMEM mistake shows up as an O(1) error.  The loose check compares against the unrounded FP64
solution within the BF16 rounding budget.
"""
from __future__ import annotations

import numpy as np
import pytest

import cuda_als_gb300 as ca
from conftest import random_csr
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL_BF16_INPUTS = 5e-4   # GPU vs FP64 oracle on BF16-rounded factors (FP32 accumulation of up
                         # to thousands of products per Gram entry, exact-solve modes)
TOL_BF16_RMSE = 2e-3     # test RMSE, BF16 vs plain FP32 after training


def bf16_round(a):
    """IEEE round-to-nearest-even to bfloat16, returned as float32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def rel_rows(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    num = np.linalg.norm(a - b, axis=1)
    den = np.maximum(np.linalg.norm(b, axis=1), 1e-6)
    return float((num / den).max())


def make_model(m, n, ptr, idx, val, f, lam=0.05, iters=1, solve=ca.SOLVE_TYPE.CHOLESKY,
               test=None, **opt):
    tr = ca.host_sparse_matrix(m, n, len(idx)).set_csr(ptr, idx, val)
    te = None if test is None else ca.host_sparse_matrix(m, n, len(test[2])).set_coo(*test)
    opt.setdefault("precision", int(ca.PRECISION.BF16))
    return ca.als_model(tr, te, f, lam, iters, ca.CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR_TENSOR,
                        solve, **opt)


def stage_boundary_problem(f, seed=0):
    """Row degrees that hit every stage edge (1, 15, 16, 17, 63, 64, 65, 128, 129, ...), a dense
    row, empty rows, and a skewed bulk."""
    rng = np.random.default_rng(seed + f)
    m, n = 300, 420
    special = [1, 15, 16, 17, 31, 32, 33, 63, 64, 65, 127, 128, 129, 255, 256, 257, n, 0, 0]
    bulk = np.minimum(rng.zipf(1.5, m - len(special)) + 1, n)
    degrees = np.concatenate([special, bulk])
    ptr, idx, val = random_csr(rng, m, n, degrees=degrees)
    return rng, m, n, ptr, idx, val


@pytest.mark.parametrize("f", [1, 10, 16, 31, 64, 100, 127, 128])
def test_tc_half_sweep_matches_oracle_on_bf16_inputs(f):
    rng, m, n, ptr, idx, val = stage_boundary_problem(f)
    lam = 0.05
    U0 = (rng.standard_normal((m, f)) * 0.1).astype(np.float32)
    V0 = (rng.standard_normal((n, f)) * 0.3).astype(np.float32)
    with make_model(m, n, ptr, idx, val, f, lam) as mdl:
        mdl.set_factors(U0, V0)
        mdl.half_sweep(0)
        U, _ = mdl.get_factors()
        assert mdl.counters()["flagged_rows"] == 0
        mdl.half_sweep(1)
        _, V = mdl.get_factors()
    # U side: the oracle on the BF16-rounded V the tensor cores saw
    Ue = U0.copy()
    O.half_sweep(ptr, idx, val, bf16_round(V0), Ue, f, lam, solve=O.CHOLESKY)
    assert rel_rows(U, Ue) < TOL_BF16_INPUTS
    assert not U[np.diff(ptr) == 0].any()  # the empty rows
    # V side (GPU-built CSC) given the GPU's U, rounded to BF16
    cptr, ridx, cval = O.csr_to_csc(m, n, ptr, idx, val)
    Ve = V0.copy()
    O.half_sweep(cptr, ridx, cval, bf16_round(U), Ve, f, lam, solve=O.CHOLESKY)
    assert rel_rows(V, Ve) < TOL_BF16_INPUTS
    # and against the unrounded FP64 solution: within the BF16 budget
    Uf = U0.copy()
    O.half_sweep(ptr, idx, val, V0, Uf, f, lam, solve=O.CHOLESKY)
    assert np.linalg.norm(U - Uf) / np.linalg.norm(Uf) < 2e-2


@pytest.mark.parametrize("solve,f", [(ca.SOLVE_TYPE.LU, 100), (ca.SOLVE_TYPE.CUMF_ALS_CG_FP32, 40),
                                     (ca.SOLVE_TYPE.CUMF_ALS_CG_FP32, 64),
                                     (ca.SOLVE_TYPE.CUMF_ALS_CG_FP32, 70),
                                     (ca.SOLVE_TYPE.CUMF_ALS_CG_FP32, 90),
                                     (ca.SOLVE_TYPE.CUMF_ALS_CG_FP32, 100),
                                     (ca.SOLVE_TYPE.CUMF_ALS_CG_FP32, 112),
                                     (ca.SOLVE_TYPE.CUMF_ALS_CG_FP32, 113),
                                     (ca.SOLVE_TYPE.CUMF_ALS_CG_FP32, 120),
                                     (ca.SOLVE_TYPE.CUMF_ALS_CG_FP32, 128),
                                     (ca.SOLVE_TYPE.LU, 128)])
def test_tc_other_solvers(solve, f):
    """LU and the FP32 CG on the tensor-core path against the oracle.  f = 40, 64 pad to 64 and
    f = 70, 90, 100, 112 to 112 (the quad-blocked CG, four groups), with 48 / 64 and 80 / 96 / 112
    Gram columns; f = 113, 120, 128 pad to 128 (quad-blocked, three groups on 160-column
    accumulators)."""
    rng, m, n, ptr, idx, val = stage_boundary_problem(f, seed=7)
    U0 = (rng.standard_normal((m, f)) * 0.1).astype(np.float32)
    V0 = (rng.standard_normal((n, f)) * 0.3).astype(np.float32)
    with make_model(m, n, ptr, idx, val, f, solve=solve, cg_tol=0.0) as mdl:
        mdl.set_factors(U0, V0)
        mdl.half_sweep(0)
        U, _ = mdl.get_factors()
    osolve = O.LU if solve == ca.SOLVE_TYPE.LU else O.CG_FP32
    Ue = U0.copy()
    O.half_sweep(ptr, idx, val, bf16_round(V0), Ue, f, 0.05, solve=osolve, cg_tol=0.0)
    tol = TOL_BF16_INPUTS if osolve == O.LU else 1e-3
    assert rel_rows(U, Ue) < tol


def _exact_factors(rng, rows, f):
    """Factor values k / 8 (|k| <= 6): exact in BF16, and every Gram entry, right-hand side and
    lambda n_u (lambda = 1/16) built from them is exact in FP32."""
    return (rng.integers(-6, 7, (rows, f)) / 8.0).astype(np.float32)


@pytest.mark.parametrize("f", [1, 10, 16, 31, 64, 100, 127, 128])
def test_tc_cg_fp16_runs_its_products_on_the_tensor_core(f):
    """Solve type 1 on the tensor-core path: CG on the regularised Gram rounded to binary16's
    significand (the reference's FP16-Gram CG, cg.cu:236-300) with every product A p on tcgen05
    (f16, the scaled Gram from TMEM), against the oracle's FP16-Gram CG, all six steps (cg_tol = 0), both
    sides.  Rounding A to 11 significant bits is discontinuous, so the inputs are chosen to make
    the regularised Gram exact in FP32: GPU and oracle then round the same matrix, and what is
    left is FP32 against FP64 vector arithmetic (the FP32-CG tolerance)."""
    rng, m, n, ptr, idx, val = stage_boundary_problem(f, seed=11)
    lam = 1.0 / 16
    U0, V0 = _exact_factors(rng, m, f), _exact_factors(rng, n, f)
    with make_model(m, n, ptr, idx, val, f, lam, solve=ca.SOLVE_TYPE.CUMF_ALS_CG_FP16,
                    cg_tol=0.0) as mdl:
        mdl.set_factors(U0, V0)
        mdl.half_sweep(0)
        U, _ = mdl.get_factors()
        assert mdl.counters()["flagged_rows"] == 0
        mdl.set_factors(U0, V0)
        mdl.half_sweep(1)
        _, V = mdl.get_factors()
    Ue = U0.copy()
    O.half_sweep(ptr, idx, val, V0, Ue, f, lam, solve=O.CG_FP16, cg_tol=0.0)
    assert rel_rows(U, Ue) < 1e-3
    assert not U[np.diff(ptr) == 0].any()
    cptr, ridx, cval = O.csr_to_csc(m, n, ptr, idx, val)
    Ve = V0.copy()
    O.half_sweep(cptr, ridx, cval, U0, Ve, f, lam, solve=O.CG_FP16, cg_tol=0.0)
    assert rel_rows(V, Ve) < 1e-3


def test_tc_cg_fp16_on_general_factors():
    """The same on unrounded factors (f = 100): where the FP32 and FP64 Grams straddle an 11-bit
    rounding boundary an entry differs by 2^-11, which CG carries into the row's solution, so the
    rows are compared in bulk (an operand-layout mistake is O(1) everywhere)."""
    f = 100
    rng, m, n, ptr, idx, val = stage_boundary_problem(f, seed=11)
    U0 = (rng.standard_normal((m, f)) * 0.1).astype(np.float32)
    V0 = (rng.standard_normal((n, f)) * 0.3).astype(np.float32)
    with make_model(m, n, ptr, idx, val, f, solve=ca.SOLVE_TYPE.CUMF_ALS_CG_FP16,
                    cg_tol=0.0) as mdl:
        mdl.set_factors(U0, V0)
        mdl.half_sweep(0)
        U, _ = mdl.get_factors()
    Ue = U0.copy()
    O.half_sweep(ptr, idx, val, bf16_round(V0), Ue, f, 0.05, solve=O.CG_FP16, cg_tol=0.0)
    d = np.asarray(U, np.float64) - Ue
    assert np.linalg.norm(d) / np.linalg.norm(Ue) < 2e-3
    assert rel_rows(U, Ue) < 5e-2


def test_tc_heavy_rows_many_stages():
    """A few rows with thousands of ratings (hundreds of pipeline stages) next to tiny rows."""
    rng = np.random.default_rng(3)
    m, n, f = 64, 6000, 100
    degrees = rng.integers(1, 40, m)
    degrees[:4] = [5999, 4096, 3000, 2049]
    ptr, idx, val = random_csr(rng, m, n, degrees=degrees)
    V0 = (rng.standard_normal((n, f)) * 0.2).astype(np.float32)
    with make_model(m, n, ptr, idx, val, f) as mdl:
        mdl.set_factors(np.zeros((m, f), np.float32), V0)
        mdl.half_sweep(0)
        U, _ = mdl.get_factors()
    Ue = np.zeros((m, f), np.float32)
    O.half_sweep(ptr, idx, val, bf16_round(V0), Ue, f, 0.05, solve=O.CHOLESKY)
    assert rel_rows(U, Ue) < TOL_BF16_INPUTS


def test_tc_training_rmse_close_to_fp32():
    """Workload 1 shape, 10 iterations: BF16 Gram test RMSE within 2e-3 of plain FP32."""
    tr, te, info = ca.synth_generate(1)
    m, n, f, lam = info["m"], info["n"], info["f"], info["lambda"]
    out = {}
    for prec in (ca.PRECISION.FP32, ca.PRECISION.BF16):
        mdl = ca.als_model(tr, te, f, lam, 10, ca.CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR,
                           ca.SOLVE_TYPE.CHOLESKY, precision=int(prec))
        mdl.train()
        out[prec] = mdl.rsme_test()
        mdl.close()
    assert abs(out[ca.PRECISION.BF16] - out[ca.PRECISION.FP32]) < TOL_BF16_RMSE


def test_tc_scaled_config3_both_sides():
    """Scaled Netflix-shaped workload (f = 100): both half-sweeps, two iterations."""
    tr, te, info = ca.synth_generate(3, scale=0.05)
    m, n, f, lam = info["m"], info["n"], info["f"], info["lambda"]
    ptr, idx, val = tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals
    with ca.als_model(tr, te, f, lam, 1, ca.CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR_TENSOR,
                      ca.SOLVE_TYPE.CHOLESKY) as mdl:
        mdl.init_factors()
        _, V0 = mdl.get_factors()
        mdl.iterate(1)
        U1, V1 = mdl.get_factors()
        assert mdl.counters()["flagged_rows"] == 0
    U0 = np.zeros((m, f), np.float32)
    O.half_sweep(ptr, idx, val, bf16_round(V0), U0, f, lam, solve=O.CHOLESKY)
    assert rel_rows(U1, U0) < TOL_BF16_INPUTS
    cptr, ridx, cval = O.csr_to_csc(m, n, ptr, idx, val)
    Ve = V0.copy()
    O.half_sweep(cptr, ridx, cval, bf16_round(U1), Ve, f, lam, solve=O.CHOLESKY)
    assert rel_rows(V1, Ve) < TOL_BF16_INPUTS
