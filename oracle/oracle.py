"""numpy front-end of the C oracle (als_oracle.c).  TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this module; it is the
checker, never the thing measured or shipped.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

_lib = None

LU, CG_FP16, CG_FP32, CHOLESKY = 0, 1, 2, 3


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        i64, i32, dbl = C.c_int64, C.c_int, C.c_double
        P = C.c_void_p
        L.oracle_init_factors.argtypes = [i64, i64, i32, P, P]
        L.oracle_half_sweep.argtypes = [i64, i32, dbl, P, P, P, P, P, i32, i32, dbl, i32, i32, P, i64]
        L.oracle_half_sweep.restype = i64
        L.oracle_train.argtypes = [i64, i64, i32, dbl, i32, P, P, P, P, P, P, i32, i32, dbl, i32, i32, P, P]
        L.oracle_train.restype = i64
        L.oracle_rmse.argtypes = [i64, P, P, P, P, P, i32]
        L.oracle_rmse.restype = dbl
        L.oracle_csr_to_csc.argtypes = [i64, i64, P, P, P, P, P, P]
        L.oracle_degree_order.argtypes = [i64, P, P]
        L.oracle_user_adjoint.argtypes = [i64, i64, i32, dbl, P, P, P, P, i64, P, P, P, P, P, P, i32]
        L.oracle_user_adjoint.restype = dbl
        L.oracle_user_loss.argtypes = [i64, i64, i32, dbl, P, P, P, P, i64, P, P, P, i32]
        L.oracle_user_loss.restype = dbl
        L.oracle_user_loss_rows.argtypes = [i64, i64, i32, dbl, P, P, P, P, i64, P, P, P, P, i32]
        L.oracle_user_loss_rows.restype = dbl
        L.oracle_max_threads.restype = i32
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def init_factors(m: int, n: int, f: int):
    """srand(0) init of als_model.cu:1772-1777 -> (U zeros m*f, V n*f)."""
    U = np.zeros((m, f), np.float32)
    V = np.zeros((n, f), np.float32)
    lib().oracle_init_factors(m, n, f, _p(U), _p(V))
    return U, V


def half_sweep(ptr, idx, val, Y, X, f, lam, solve=LU, cg_iters=6, cg_tol=1e-4, fp32=False,
               threads=0, rows_subset=None):
    """Solve every row (or rows_subset) in place into X; returns the flagged-row count."""
    ptr, idx, val = _c(ptr, np.int32), _c(idx, np.int32), _c(val, np.float32)
    Y = _c(Y, np.float32)
    assert X.dtype == np.float32 and X.flags.c_contiguous
    sub = None if rows_subset is None else _c(rows_subset, np.int32)
    return int(lib().oracle_half_sweep(len(ptr) - 1, f, lam, _p(ptr), _p(idx), _p(val), _p(Y),
                                       _p(X), solve, cg_iters, cg_tol, 1 if fp32 else 0, threads,
                                       _p(sub), 0 if sub is None else len(sub)))


def train(m, n, f, lam, iters, csr, csc, solve=LU, cg_iters=6, cg_tol=1e-4, fp32=False,
          threads=0):
    """init + iters x (U half over the CSR, V half over the CSC) -> (U, V, flagged)."""
    U = np.zeros((m, f), np.float32)
    V = np.zeros((n, f), np.float32)
    cp, ci, cv = (_c(csr[0], np.int32), _c(csr[1], np.int32), _c(csr[2], np.float32))
    tp, ti, tv = (_c(csc[0], np.int32), _c(csc[1], np.int32), _c(csc[2], np.float32))
    flagged = lib().oracle_train(m, n, f, lam, iters, _p(cp), _p(ci), _p(cv), _p(tp), _p(ti),
                                 _p(tv), solve, cg_iters, cg_tol, 1 if fp32 else 0, threads,
                                 _p(U), _p(V))
    return U, V, int(flagged)


def rmse(rows, cols, vals, U, V) -> float:
    rows, cols, vals = _c(rows, np.int32), _c(cols, np.int32), _c(vals, np.float32)
    U, V = _c(U, np.float32), _c(V, np.float32)
    return float(lib().oracle_rmse(len(vals), _p(rows), _p(cols), _p(vals), _p(U), _p(V),
                                   U.shape[1]))


def csr_to_csc(rows, cols, ptr, idx, val):
    ptr, idx, val = _c(ptr, np.int32), _c(idx, np.int32), _c(val, np.float32)
    cptr = np.zeros(cols + 1, np.int32)
    ridx = np.zeros(len(idx), np.int32)
    cval = np.zeros(len(idx), np.float32)
    lib().oracle_csr_to_csc(rows, cols, _p(ptr), _p(idx), _p(val), _p(cptr), _p(ridx), _p(cval))
    return cptr, ridx, cval


def degree_order(ptr):
    ptr = _c(ptr, np.int32)
    perm = np.zeros(len(ptr) - 1, np.int32)
    lib().oracle_degree_order(len(ptr) - 1, _p(ptr), _p(perm))
    return perm


def user_adjoint(m, n, f, lam, csr, Y, held, threads=0):
    """FP64 forward user half-sweep, held-out loss and gradient -> (loss, X, dLdY, dLdlambda)."""
    cp, ci, cv = (_c(csr[0], np.int32), _c(csr[1], np.int32), _c(csr[2], np.float32))
    Y = _c(Y, np.float64)
    hr, hc, hv = (_c(held[0], np.int32), _c(held[1], np.int32), _c(held[2], np.float32))
    X = np.zeros((m, f), np.float64)
    G = np.zeros((n, f), np.float64)
    dl = C.c_double(0.0)
    loss = lib().oracle_user_adjoint(m, n, f, lam, _p(cp), _p(ci), _p(cv), _p(Y), len(hv),
                                     _p(hr), _p(hc), _p(hv), _p(X), _p(G), C.byref(dl), threads)
    return float(loss), X, G, float(dl.value)


def user_loss(m, n, f, lam, csr, Y, held, threads=0) -> float:
    cp, ci, cv = (_c(csr[0], np.int32), _c(csr[1], np.int32), _c(csr[2], np.float32))
    Y = _c(Y, np.float64)
    hr, hc, hv = (_c(held[0], np.int32), _c(held[1], np.int32), _c(held[2], np.float32))
    return float(lib().oracle_user_loss(m, n, f, lam, _p(cp), _p(ci), _p(cv), _p(Y), len(hv),
                                        _p(hr), _p(hc), _p(hv), threads))


def user_loss_rows(m, n, f, lam, csr, Y, held, row_mask, threads=0) -> float:
    """Held-out loss of the FP64 user half-sweep restricted to the rows in row_mask."""
    cp, ci, cv = (_c(csr[0], np.int32), _c(csr[1], np.int32), _c(csr[2], np.float32))
    Y = _c(Y, np.float64)
    hr, hc, hv = (_c(held[0], np.int32), _c(held[1], np.int32), _c(held[2], np.float32))
    mask = _c(row_mask, np.uint8)
    return float(lib().oracle_user_loss_rows(m, n, f, lam, _p(cp), _p(ci), _p(cv), _p(Y), len(hv),
                                             _p(hr), _p(hc), _p(hv), _p(mask), threads))


def rows_touching(m, csr, held, item):
    """Rows whose training ratings or held-out ratings involve `item`."""
    ptr, idx = np.asarray(csr[0]), np.asarray(csr[1])
    rows = np.repeat(np.arange(m, dtype=np.int64), np.diff(ptr))
    mask = np.zeros(m, np.uint8)
    mask[rows[idx == item]] = 1
    mask[np.asarray(held[0])[np.asarray(held[1]) == item]] = 1
    return mask
