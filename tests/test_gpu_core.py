"""GPU parity through the C ABI: index kernels bit-exact, FP32 sweeps within tolerance of the
FP64 oracle, RMSE, the reference-shaped model API and its error paths."""
from __future__ import annotations

import numpy as np
import pytest
import scipy.sparse as sp

import cuda_als_gb300 as ca
from conftest import load_toy, random_csr
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# Tolerances of the FP32 path against the FP64 oracle (relative, row-norm-wise for factors).
TOL_SOLVE = 1e-4     # one half-sweep with an exact solver (LU / Cholesky)
TOL_CG = 1e-3        # one half-sweep of 6-step CG (FP32 vs FP64 iterates)
TOL_TRAIN = 1e-4     # factors after training (relative Frobenius)
TOL_RMSE = 1e-4      # test RMSE after training (absolute)


def model_from_csr(m, n, ptr, idx, val, f, lam=0.05, iters=1, test=None, csc=None, **opt):
    tr = ca.host_sparse_matrix(m, n, len(idx)).set_csr(ptr, idx, val)
    if csc is not None:
        tr.set_csc(*csc)
    te = None
    if test is not None:
        te = ca.host_sparse_matrix(m, n, len(test[2])).set_coo(*test)
    opt.setdefault("calculate_vtvs_type", ca.CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR)
    opt.setdefault("solve_type", ca.SOLVE_TYPE.LU)
    vt, st = opt.pop("calculate_vtvs_type"), opt.pop("solve_type")
    return ca.als_model(tr, te, f, lam, iters, vt, st, **opt)


def rel_rows(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    num = np.linalg.norm(a - b, axis=1)
    den = np.maximum(np.linalg.norm(b, axis=1), 1e-6)
    return float((num / den).max())


# ---------------------------------------------------------------- index kernels (bit-exact)

def test_gpu_transpose_matches_reference_prep_logs(toy):
    cptr, ridx, cval = ca.csr_to_csc(toy["m"], toy["n"], toy["R_train_csr_indptr"],
                                     toy["R_train_csr_indices"], toy["R_train_csr_data"])
    assert np.array_equal(cptr, toy["R_train_csc_indptr"])
    assert np.array_equal(ridx, toy["R_train_csc_indices"])
    assert np.array_equal(cval, toy["R_train_csc_data"].astype(np.float32))


@pytest.mark.parametrize("case", ["cfg1", "cfg3", "cfg4", "wide", "narrow", "empty", "one_row",
                                  "nnz0"])
def test_gpu_transpose_bit_exact(case):
    rng = np.random.default_rng(1)
    if case.startswith("cfg"):
        k = int(case[3:])
        tr, _, info = ca.synth_generate(k, scale=1.0 if k == 1 else 0.04)
        m, n = info["m"], info["n"]
        ptr, idx, val = tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals
    elif case == "wide":   # > 2^16 columns: three radix passes
        m, n = 300, 150000
        ptr, idx, val = random_csr(rng, m, n, density=0.002, values=(0, 9))
    elif case == "narrow":  # <= 256 columns: one radix pass straight into the CSC arrays
        m, n = 3000, 200
        ptr, idx, val = random_csr(rng, m, n, density=0.05)
    elif case == "empty":  # empty rows and empty columns
        m, n = 200, 700
        ptr, idx, val = random_csr(rng, m, n, density=0.01, empty_rows=set(range(0, 200, 3)))
    elif case == "one_row":
        m, n = 1, 5000
        ptr, idx, val = random_csr(rng, m, n, density=0.3)
    else:
        m, n = 10, 10
        ptr, idx, val = np.zeros(11, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32)
    cptr, ridx, cval = ca.csr_to_csc(m, n, ptr, idx, val)
    e_ptr, e_idx, e_val = O.csr_to_csc(m, n, ptr, idx, val)
    assert np.array_equal(cptr, e_ptr)
    assert np.array_equal(ridx, e_idx)
    assert np.array_equal(cval, e_val)
    if len(idx):
        ref = sp.csr_matrix((val, idx, ptr), shape=(m, n)).tocsc()
        assert np.array_equal(cptr, ref.indptr) and np.array_equal(ridx, ref.indices)


@pytest.mark.parametrize("kind", ["synthetic", "ties", "big_degrees"])
def test_gpu_degree_order_bit_exact(kind):
    rng = np.random.default_rng(2)
    if kind == "synthetic":
        ptr = ca.synth_generate(3, scale=0.04)[0].h_csr_row_ptrs
    elif kind == "ties":
        ptr = np.concatenate([[0], np.cumsum(rng.integers(0, 3, 10000))]).astype(np.int32)
    else:
        ptr = np.concatenate([[0], np.cumsum(rng.integers(0, 300000, 50))]).astype(np.int32)
    assert np.array_equal(ca.degree_order(ptr), O.degree_order(ptr))


# ---------------------------------------------------------------- FP32 half-sweeps vs FP64

def _skewed_problem(f):
    rng = np.random.default_rng(100 + f)
    m, n = 400, 300
    degrees = np.minimum(rng.zipf(1.6, m) + 3, n)
    degrees[:3] = [n, n // 2, 1]   # a dense row, a heavy row and a single-rating row
    ptr, idx, val = random_csr(rng, m, n, degrees=degrees)
    return rng, m, n, ptr, idx, val


@pytest.mark.parametrize("f", [1, 10, 20, 64, 100, 128])
@pytest.mark.parametrize("solve", [ca.SOLVE_TYPE.LU, ca.SOLVE_TYPE.CHOLESKY,
                                   ca.SOLVE_TYPE.CUMF_ALS_CG_FP32])
def test_gpu_half_sweep_fp32_matches_oracle(f, solve):
    """Both half-sweeps from the same inputs.  CG runs its 6 steps without the early exit
    (cg_tol = 0) so FP32 and FP64 follow the same iteration path."""
    rng, m, n, ptr, idx, val = _skewed_problem(f)
    lam = 0.05
    cg_tol = 0.0
    with model_from_csr(m, n, ptr, idx, val, f, lam, solve_type=solve, cg_tol=cg_tol) as mdl:
        U0 = (rng.standard_normal((m, f)) * 0.1).astype(np.float32)
        V0 = (rng.standard_normal((n, f)) * 0.3).astype(np.float32)
        mdl.set_factors(U0, V0)
        mdl.half_sweep(0)
        U, _ = mdl.get_factors()
        assert mdl.counters()["flagged_rows"] == 0
        # the V side uses the GPU-built CSC
        mdl.half_sweep(1)
        _, V = mdl.get_factors()
    osolve = {0: O.LU, 3: O.CHOLESKY, 2: O.CG_FP32}[int(solve)]
    Ue = U0.copy()
    O.half_sweep(ptr, idx, val, V0, Ue, f, lam, solve=osolve, cg_tol=cg_tol)
    cptr, ridx, cval = O.csr_to_csc(m, n, ptr, idx, val)
    Ve = V0.copy()
    O.half_sweep(cptr, ridx, cval, U, Ve, f, lam, solve=osolve, cg_tol=cg_tol)
    if osolve != O.CG_FP32:
        assert rel_rows(U, Ue) < TOL_SOLVE
        assert rel_rows(V, Ve) < TOL_SOLVE
    else:
        # U-side systems are well conditioned: the FP32 iterates follow FP64's.  On the V side a
        # 6-step CG that has converged keeps stepping on rounding noise (in FP32 and FP64 alike,
        # with different noise), so only the residual is comparable there.
        assert rel_rows(U, Ue) < TOL_CG
        bn = _rhs_norms(cptr, ridx, cval, U)
        rg = np.sqrt(_residuals(cptr, ridx, cval, U, V, f, lam) / bn).max()
        re = np.sqrt(_residuals(cptr, ridx, cval, U, Ve, f, lam) / bn).max()
        assert rg <= 4 * re + 1e-2


def _rhs_norms(ptr, idx, val, Y):
    out = np.zeros(len(ptr) - 1)
    for u in range(len(ptr) - 1):
        cols = idx[ptr[u]:ptr[u + 1]]
        b = Y[cols].astype(np.float64).T @ val[ptr[u]:ptr[u + 1]]
        out[u] = b @ b
    return out


def _residuals(ptr, idx, val, Y, X, f, lam):
    out = np.zeros(len(ptr) - 1)
    for u in range(len(ptr) - 1):
        cols = idx[ptr[u]:ptr[u + 1]]
        Yu = Y[cols].astype(np.float64)
        A = Yu.T @ Yu + lam * len(cols) * np.eye(f)
        r = Yu.T @ val[ptr[u]:ptr[u + 1]] - A @ X[u].astype(np.float64)
        out[u] = r @ r
    return out


@pytest.mark.parametrize("f", [20, 100])
def test_gpu_cg_exit_rule_matches_reference_semantics(f):
    """With the reference's exit rule (r'r < 1e-4 after a step, cg.cu:196) a row may stop one
    step earlier or later in FP32 than in FP64; every GPU row must still end either below the
    tolerance or after all 6 steps with a residual no worse than 4x the FP64 run's."""
    rng, m, n, ptr, idx, val = _skewed_problem(f)
    cptr, ridx, cval = O.csr_to_csc(m, n, ptr, idx, val)
    U0 = (rng.standard_normal((m, f)) * 0.1).astype(np.float32)
    V0 = (rng.standard_normal((n, f)) * 0.3).astype(np.float32)
    with model_from_csr(m, n, ptr, idx, val, f, 0.05,
                        solve_type=ca.SOLVE_TYPE.CUMF_ALS_CG_FP32) as mdl:
        mdl.set_factors(U0, V0)
        mdl.half_sweep(1)
        _, V = mdl.get_factors()
    Ve = V0.copy()
    O.half_sweep(cptr, ridx, cval, U0, Ve, f, 0.05, solve=O.CG_FP32)
    rg = _residuals(cptr, ridx, cval, U0, V, f, 0.05)
    re = _residuals(cptr, ridx, cval, U0, Ve, f, 0.05)
    assert np.all((rg < 2e-4) | (rg <= 4 * re + 1e-6))
    close = np.linalg.norm(V - Ve, axis=1) <= 1e-3 * np.maximum(np.linalg.norm(Ve, axis=1), 1e-6)
    assert close.mean() > 0.9


def test_gpu_cg_fp16_mode_runs_close_to_fp32_cg():
    rng = np.random.default_rng(5)
    m, n, f = 200, 150, 32
    ptr, idx, val = random_csr(rng, m, n, density=0.1)
    V0 = (rng.standard_normal((n, f)) * 0.3).astype(np.float32)
    out = {}
    for st in (ca.SOLVE_TYPE.CUMF_ALS_CG_FP16, ca.SOLVE_TYPE.CUMF_ALS_CG_FP32):
        with model_from_csr(m, n, ptr, idx, val, f, solve_type=st) as mdl:
            mdl.set_factors(np.zeros((m, f), np.float32), V0)
            mdl.half_sweep(0)
            out[int(st)] = mdl.get_factors()[0]
    Ue = np.zeros((m, f), np.float32)
    O.half_sweep(ptr, idx, val, V0, Ue, f, 0.05, solve=O.CG_FP16)
    assert rel_rows(out[1], Ue) < 1e-2
    assert rel_rows(out[1], out[2]) < 1e-2


# ---------------------------------------------------------------- training parity

def _synthetic(k, scale):
    tr, te, info = ca.synth_generate(k, scale=scale)
    csr = (tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals)
    test = (te.h_coo_row_idxs, te.h_csr_coo_col_idxs, te.h_csr_coo_vals)
    return info, csr, test


@pytest.mark.parametrize("solve", [ca.SOLVE_TYPE.LU, ca.SOLVE_TYPE.CHOLESKY])
def test_gpu_train_config1_matches_oracle(solve):
    """Config 1 (1000 x 500, 20k ratings, f=10, lambda=0.05, 10 iterations, per-row exact solve)."""
    info, csr, test = _synthetic(1, 1.0)
    m, n, f, lam = info["m"], info["n"], info["f"], info["lambda"]
    with model_from_csr(m, n, *csr, f, lam, iters=10, test=test, solve_type=solve) as mdl:
        mdl.train()
        U, V = mdl.h_UT, mdl.h_VT
        rmse = mdl.rsme_test()
    csc = O.csr_to_csc(m, n, *csr)
    Ue, Ve, flagged = O.train(m, n, f, lam, 10, csr, csc, solve=O.LU)
    assert flagged == 0
    assert np.linalg.norm(U - Ue) / np.linalg.norm(Ue) < TOL_TRAIN
    assert np.linalg.norm(V - Ve) / np.linalg.norm(Ve) < TOL_TRAIN
    rmse_e = O.rmse(*test, Ue, Ve)
    assert abs(rmse - rmse_e) < TOL_RMSE
    assert abs(rmse - O.rmse(*test, U, V)) < 1e-12


def test_gpu_reference_style_usage_on_toy_files(tmp_path, toy):
    """main.cpp:68-105 through the mirror classes: .bin loads -> als_model -> train -> RMSE."""
    from test_abi import _write_dataset

    _write_dataset(tmp_path, toy)
    m, n = toy["m"], toy["n"]
    nnz, nt = len(toy["R_train_csr_data"]), len(toy["R_test_coo_data"])
    f = 100 if toy["m"] == 15 else 20   # config/toy_data.ini, config/toy_data_2.ini
    tr, te = ca.load_dataset(str(tmp_path), m, n, nnz, nt)
    model = ca.als_model(tr, te, f, 0.05, 10, ca.CALCULATE_VTVS_TYPE.SIMPLE, ca.SOLVE_TYPE.LU,
                         32, 1, 1)
    model.train()
    csr = (toy["R_train_csr_indptr"], toy["R_train_csr_indices"], toy["R_train_csr_data"])
    csc = (toy["R_train_csc_indptr"], toy["R_train_csc_indices"], toy["R_train_csc_data"])
    Ue, Ve, _ = O.train(m, n, f, 0.05, 10, csr, csc, solve=O.LU)
    assert np.linalg.norm(model.h_UT - Ue) / np.linalg.norm(Ue) < TOL_TRAIN
    assert np.linalg.norm(model.h_VT - Ve) / np.linalg.norm(Ve) < TOL_TRAIN
    test = (toy["R_test_coo_row"], toy["R_test_coo_col"], toy["R_test_coo_data"])
    assert abs(model.rsme_test() - O.rmse(*test, Ue, Ve)) < TOL_RMSE
    coo_rows = np.repeat(np.arange(m), np.diff(csr[0]))
    assert abs(model.rsme_train() - O.rmse(coo_rows, csr[1], csr[2], Ue, Ve)) < TOL_RMSE
    # save_libmf (als_model.cu:2294-2312)
    model.save_libmf(str(tmp_path / "model.bin"))
    raw = (tmp_path / "model.bin").read_bytes()
    hdr = np.frombuffer(raw[:16], np.int32)
    assert list(hdr) == [0, m, n, f]
    mean = np.frombuffer(raw[16:20], np.float32)[0]
    assert mean == pytest.approx(float(np.mean(csr[2])), rel=1e-6)
    body = np.frombuffer(raw[20:], np.float32)
    assert np.array_equal(body[:m * f], model.h_UT.ravel())
    assert np.array_equal(body[m * f:], model.h_VT.ravel())
    model.close()


def test_gpu_uploaded_csc_equals_built_csc():
    info, csr, test = _synthetic(1, 1.0)
    m, n, f = info["m"], info["n"], 10
    csc = O.csr_to_csc(m, n, *csr)
    res = []
    for give in (False, True):
        with model_from_csr(m, n, *csr, f, iters=3, test=test, csc=csc if give else None) as mdl:
            mdl.train()
            res.append((mdl.h_UT.copy(), mdl.h_VT.copy(), mdl.rsme_test()))
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])
    assert res[0][2] == res[1][2]


def test_gpu_update_values_refreshes_both_layouts():
    info, csr, test = _synthetic(1, 1.0)
    m, n, f = info["m"], info["n"], 10
    new_vals = (6.0 - csr[2]).astype(np.float32)
    with model_from_csr(m, n, *csr, f, iters=2) as mdl:
        mdl.update_values(new_vals)
        mdl.train()
        U, V = mdl.h_UT.copy(), mdl.h_VT.copy()
    with model_from_csr(m, n, csr[0], csr[1], new_vals, f, iters=2) as mdl:
        mdl.train()
        assert np.array_equal(U, mdl.h_UT) and np.array_equal(V, mdl.h_VT)


# ---------------------------------------------------------------- RMSE

def test_gpu_rmse_deterministic_and_matches_oracle():
    info, csr, test = _synthetic(3, 0.04)
    m, n, f = info["m"], info["n"], 16
    rng = np.random.default_rng(9)
    U = rng.standard_normal((m, f)).astype(np.float32)
    V = rng.standard_normal((n, f)).astype(np.float32)
    U[5, 3] = np.nan   # the NaN rule: the dot stops at the NaN component
    with model_from_csr(m, n, *csr, f, test=test) as mdl:
        mdl.set_factors(U, V)
        a, b = mdl.rsme_test(), mdl.rsme_test()
        assert a == b
        assert a == pytest.approx(O.rmse(*test, U, V), rel=1e-12)
        rows = np.repeat(np.arange(m), np.diff(csr[0]))
        assert mdl.rsme_train() == pytest.approx(O.rmse(rows, csr[1], csr[2], U, V), rel=1e-12)


# ---------------------------------------------------------------- errors and edge rows

def test_gpu_invalid_inputs_are_rejected():
    rng = np.random.default_rng(4)
    ptr, idx, val = random_csr(rng, 50, 40, density=0.2)
    bad = idx.copy()
    bad[7] = 40
    with pytest.raises(ca.ALSError) as e:
        model_from_csr(50, 40, ptr, bad, val, 8)
    assert e.value.status == ca.Status.INVALID_ARG
    nanv = val.copy()
    nanv[3] = np.nan
    with pytest.raises(ca.ALSError):
        model_from_csr(50, 40, ptr, idx, nanv, 8)
    badp = ptr.copy()
    badp[10] = badp[11] + 1
    with pytest.raises(ca.ALSError):
        model_from_csr(50, 40, badp, idx, val, 8)
    with pytest.raises(ca.ALSError):
        model_from_csr(50, 40, ptr, idx, val, 0)
    with pytest.raises(ca.ALSError):
        model_from_csr(50, 40, ptr, idx, val, 8, solve_type=9)
    test = (np.array([0, 50], np.int32), np.array([1, 2], np.int32), np.ones(2, np.float32))
    with pytest.raises(ca.ALSError):
        model_from_csr(50, 40, ptr, idx, val, 8, test=test)


def test_gpu_empty_rows_and_columns_solve_to_zero():
    rng = np.random.default_rng(6)
    m, n, f = 60, 50, 8
    ptr, idx, val = random_csr(rng, m, n, density=0.1, empty_rows={0, 7, 59})
    idx = np.where(idx == 3, 4, idx).astype(np.int32)   # column 3 empty (duplicates are fine)
    with model_from_csr(m, n, ptr, idx, val, f, iters=2) as mdl:
        mdl.train()
        assert not mdl.h_UT[[0, 7, 59]].any()
        assert not mdl.h_VT[3].any()
        assert np.isfinite(mdl.h_UT).all() and np.isfinite(mdl.h_VT).all()


@pytest.mark.parametrize("f,solve", [(64, ca.SOLVE_TYPE.CHOLESKY), (100, ca.SOLVE_TYPE.LU),
                                     (100, ca.SOLVE_TYPE.CUMF_ALS_CG_FP32)])
def test_fp32_rows_split_into_parts_match_the_oracle(f, solve):
    """Rows above 16,384 ratings run as parts (partial Grams by separate CTAs, added in order):
    degrees on both sides of the threshold, a row of 50k ratings, light rows beside them."""
    rng = np.random.default_rng(f)
    m, n = 8, 60000
    degrees = np.array([50000, 40000, 16385, 16384, 16383, 100, 3, 0])
    ptr, idx, val = random_csr(rng, m, n, degrees=degrees)
    V0 = (rng.standard_normal((n, f)) * 0.1).astype(np.float32)
    U0 = (rng.standard_normal((m, f)) * 0.1).astype(np.float32)
    tr = ca.host_sparse_matrix(m, n, len(idx)).set_csr(ptr, idx, val)
    with ca.als_model(tr, None, f, 0.05, 1, ca.CALCULATE_VTVS_TYPE.SIMPLE, solve,
                      precision=int(ca.PRECISION.FP32), cg_tol=0.0) as mdl:
        mdl.set_factors(U0, V0)
        mdl.half_sweep(0)
        U, _ = mdl.get_factors()
        assert mdl.counters()["flagged_rows"] == 0
    osolve = {ca.SOLVE_TYPE.CHOLESKY: O.CHOLESKY, ca.SOLVE_TYPE.LU: O.LU,
              ca.SOLVE_TYPE.CUMF_ALS_CG_FP32: O.CG_FP32}[solve]
    Ue = U0.copy()
    O.half_sweep(ptr, idx, val, V0, Ue, f, 0.05, solve=osolve, cg_tol=0.0)
    num = np.linalg.norm(U.astype(np.float64) - Ue, axis=1)
    den = np.maximum(np.linalg.norm(Ue.astype(np.float64), axis=1), 1e-6)
    assert (num / den).max() < (1e-4 if osolve != O.CG_FP32 else 1e-3)
    assert not U[-1].any()
