"""The oracle against the reference's known answers and against independent math (CPU only).

Pins: the CSR->CSC transpose against the arrays the reference's toy prep scripts printed
(data/toy_data*/prepare_*.log); the init against libc rand(); the per-row solve against numpy;
the adjoint against FP64 central finite differences.
"""
from __future__ import annotations

import ctypes
import ctypes.util

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import load_toy, random_csr
from oracle import oracle as O


def test_transpose_matches_reference_prep_logs(toy):
    cptr, ridx, cval = O.csr_to_csc(toy["m"], toy["n"], toy["R_train_csr_indptr"],
                                    toy["R_train_csr_indices"], toy["R_train_csr_data"])
    assert np.array_equal(cptr, toy["R_train_csc_indptr"])
    assert np.array_equal(ridx, toy["R_train_csc_indices"])
    assert np.array_equal(cval, toy["R_train_csc_data"].astype(np.float32))


def test_transpose_matches_scipy_on_random(rng_seed=7):
    rng = np.random.default_rng(rng_seed)
    ptr, idx, val = random_csr(rng, 300, 170, density=0.05, empty_rows={3, 4, 200})
    cptr, ridx, cval = O.csr_to_csc(300, 170, ptr, idx, val)
    ref = sp.csr_matrix((val, idx, ptr), shape=(300, 170)).tocsc()
    assert np.array_equal(cptr, ref.indptr)
    assert np.array_equal(ridx, ref.indices)
    assert np.array_equal(cval, ref.data)


def test_degree_order_is_stable_descending():
    rng = np.random.default_rng(3)
    deg = rng.integers(0, 9, size=500)
    ptr = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
    perm = O.degree_order(ptr)
    assert np.array_equal(perm, np.argsort(-deg, kind="stable"))


def test_init_matches_libc_rand():
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    U, V = O.init_factors(7, 11, 5)
    libc.srand(0)
    raw = np.array([libc.rand() for _ in range(11 * 5)], dtype=np.int64)
    # als_model.cu:1775: 0.2*((float)rand()/(float)RAND_MAX)
    expect = (0.2 * (raw.astype(np.float32) / np.float32(2147483647)).astype(np.float64)).astype(
        np.float32)
    assert np.array_equal(V.ravel(), expect)
    assert not U.any()


def _dense_rows(ptr, idx, val, Y, f, lam):
    X = np.zeros((len(ptr) - 1, f))
    for u in range(len(ptr) - 1):
        cols = idx[ptr[u]:ptr[u + 1]]
        if len(cols) == 0:
            continue
        Yu = Y[cols].astype(np.float64)
        A = Yu.T @ Yu + lam * len(cols) * np.eye(f)
        X[u] = np.linalg.solve(A, Yu.T @ val[ptr[u]:ptr[u + 1]].astype(np.float64))
    return X


@pytest.mark.parametrize("solve", [O.LU, O.CHOLESKY])
@pytest.mark.parametrize("f", [1, 7, 33])
def test_half_sweep_exact_solves_match_numpy(solve, f):
    rng = np.random.default_rng(f)
    ptr, idx, val = random_csr(rng, 60, 40, density=0.2, empty_rows={5})
    Y = (rng.standard_normal((40, f)) * 0.4).astype(np.float32)
    X = np.full((60, f), 9.0, np.float32)
    flagged = O.half_sweep(ptr, idx, val, Y, X, f, 0.05, solve=solve)
    assert flagged == 0
    ref = _dense_rows(ptr, idx, val, Y, f, 0.05)
    np.testing.assert_allclose(X, ref, rtol=2e-5, atol=2e-6)
    assert not X[5].any()  # empty row -> 0


def test_cg_converges_to_exact():
    rng = np.random.default_rng(11)
    f = 12
    ptr, idx, val = random_csr(rng, 40, 30, density=0.5)
    Y = (rng.standard_normal((30, f)) * 0.4).astype(np.float32)
    X = np.zeros((40, f), np.float32)
    O.half_sweep(ptr, idx, val, Y, X, f, 0.05, solve=O.CG_FP32, cg_iters=200, cg_tol=0.0)
    np.testing.assert_allclose(X, _dense_rows(ptr, idx, val, Y, f, 0.05), rtol=1e-4, atol=1e-5)


def test_rmse_matches_numpy_and_nan_rule():
    rng = np.random.default_rng(5)
    U = rng.standard_normal((10, 4)).astype(np.float32)
    V = rng.standard_normal((8, 4)).astype(np.float32)
    rows = rng.integers(0, 10, 50).astype(np.int32)
    cols = rng.integers(0, 8, 50).astype(np.int32)
    vals = rng.integers(1, 6, 50).astype(np.float32)
    pred = np.einsum("ij,ij->i", U[rows].astype(np.float64), V[cols].astype(np.float64))
    ref = np.sqrt(np.mean((vals - pred) ** 2))
    assert O.rmse(rows, cols, vals, U, V) == pytest.approx(ref, rel=1e-12)
    # a NaN component ends the dot product there (als_model.cu:78-79)
    U2 = U.copy()
    U2[rows[0], 2] = np.nan
    partial = float(np.dot(U[rows[0], :2].astype(np.float64), V[cols[0], :2].astype(np.float64)))
    pred2 = pred.copy()
    for e in range(50):
        if rows[e] == rows[0]:
            pred2[e] = np.dot(U[rows[e], :2].astype(np.float64), V[cols[e], :2].astype(np.float64))
    assert pred2[0] == pytest.approx(partial)
    ref2 = np.sqrt(np.mean((vals - pred2) ** 2))
    assert O.rmse(rows, cols, vals, U2, V) == pytest.approx(ref2, rel=1e-12)


def test_train_reduces_toy_rmse():
    t = load_toy("toy_data_2")
    m, n, f = t["m"], t["n"], 20
    csr = (t["R_train_csr_indptr"], t["R_train_csr_indices"], t["R_train_csr_data"])
    csc = (t["R_train_csc_indptr"], t["R_train_csc_indices"], t["R_train_csc_data"])
    U, V, flagged = O.train(m, n, f, 0.05, 10, csr, csc)
    assert flagged == 0
    coo_rows = np.repeat(np.arange(m), np.diff(csr[0]))
    train_rmse = O.rmse(coo_rows, csr[1], csr[2], U, V)
    U0, V0 = O.init_factors(m, n, f)
    assert train_rmse < 0.5 * O.rmse(coo_rows, csr[1], csr[2], U0, V0)


def test_adjoint_matches_central_differences():
    """dL/dY and dL/dlambda of the held-out loss against FP64 central differences (1e-5 rel)."""
    rng = np.random.default_rng(21)
    m, n, f, lam = 25, 18, 5, 0.3
    ptr, idx, val = random_csr(rng, m, n, density=0.35)
    Y = rng.standard_normal((n, f)) * 0.5
    hr = rng.integers(0, m, 60).astype(np.int32)
    hc = rng.integers(0, n, 60).astype(np.int32)
    hv = rng.integers(1, 6, 60).astype(np.float32)
    csr, held = (ptr, idx, val), (hr, hc, hv)
    loss, X, G, dlam = O.user_adjoint(m, n, f, lam, csr, Y, held)
    assert loss == pytest.approx(O.user_loss(m, n, f, lam, csr, Y, held), rel=1e-14)
    h = 1e-5
    picks = [(int(a), int(b)) for a, b in zip(rng.integers(0, n, 16), rng.integers(0, f, 16))]
    for (i, k) in picks:
        Yp, Ym = Y.copy(), Y.copy()
        Yp[i, k] += h
        Ym[i, k] -= h
        fd = (O.user_loss(m, n, f, lam, csr, Yp, held) - O.user_loss(m, n, f, lam, csr, Ym, held)) / (2 * h)
        assert G[i, k] == pytest.approx(fd, rel=1e-5, abs=1e-8), (i, k)
    fd = (O.user_loss(m, n, f, lam + h, csr, Y, held) - O.user_loss(m, n, f, lam - h, csr, Y, held)) / (2 * h)
    assert dlam == pytest.approx(fd, rel=1e-5)


def test_adjoint_central_differences_on_workload5_shape():
    """64 random coordinates of dL/dY and dL/dlambda on a scaled MovieLens-latest-shaped workload
    (f = 128), FP64 central differences of the loss restricted to the rows each item touches."""
    import cuda_als_gb300 as ca

    tr, te, info = ca.synth_generate(5, scale=0.03)
    m, n, f, lam = info["m"], info["n"], info["f"], info["lambda"]
    csr = (tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals)
    held = (te.h_coo_row_idxs, te.h_csr_coo_col_idxs, te.h_csr_coo_vals)
    rng = np.random.default_rng(5)
    Y = rng.standard_normal((n, f)) * 0.2
    loss, X, G, dlam = O.user_adjoint(m, n, f, lam, csr, Y, held)
    h = 1e-5
    items = rng.integers(0, n, 64)
    ks = rng.integers(0, f, 64)
    for i, k in zip(items, ks):
        mask = O.rows_touching(m, csr, held, int(i))
        Yp, Ym = Y.copy(), Y.copy()
        Yp[i, k] += h
        Ym[i, k] -= h
        fd = (O.user_loss_rows(m, n, f, lam, csr, Yp, held, mask) -
              O.user_loss_rows(m, n, f, lam, csr, Ym, held, mask)) / (2 * h)
        assert G[i, k] == pytest.approx(fd, rel=1e-5, abs=1e-9), (int(i), int(k))
    fd = (O.user_loss(m, n, f, lam + h, csr, Y, held) - O.user_loss(m, n, f, lam - h, csr, Y, held)) / (2 * h)
    assert dlam == pytest.approx(fd, rel=1e-5)
