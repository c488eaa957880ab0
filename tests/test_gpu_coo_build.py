"""The GPU triples -> CSR / CSC builder (als_coo_to_csr, als_coo_to_csr_device) through the C ABI:
bit-exact against the reference's logged toy arrays, the oracle restatement and scipy, on edge
cases and on a full-size workload's shuffled triples."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import cuda_als_gb300 as ca
from conftest import load_toy
from oracle import coo as OC
from test_coo_build import random_triples

pytestmark = pytest.mark.gpu


def _same(got, want):
    (p, i, v), r, csc = got
    (wp, wi, wv), wr, (wcp, wri, wcv) = want
    assert np.array_equal(p, wp) and np.array_equal(i, wi) and np.array_equal(r, wr)
    assert np.array_equal(v.view(np.uint32), wv.view(np.uint32))
    cp, ri, cv = csc
    assert np.array_equal(cp, wcp) and np.array_equal(ri, wri)
    assert np.array_equal(cv.view(np.uint32), wcv.view(np.uint32))


@pytest.mark.parametrize("name", ["toy_data", "toy_data_2"])
def test_gpu_builder_reproduces_the_reference_logs(name):
    d = load_toy(name)
    m, n = d["m"], d["n"]
    (ptr, idx, val), crow, (cptr, ridx, cval) = ca.coo_to_csr(
        m, n, d["raw_train_row"], d["raw_train_col"], d["raw_train_val"])
    assert np.array_equal(ptr, d["R_train_csr_indptr"])
    assert np.array_equal(idx, d["R_train_csr_indices"])
    assert np.array_equal(val, d["R_train_csr_data"].astype(np.float32))
    assert np.array_equal(cptr, d["R_train_csc_indptr"])
    assert np.array_equal(ridx, d["R_train_csc_indices"])
    assert np.array_equal(cval, d["R_train_csc_data"].astype(np.float32))
    tm, tn = int(d["raw_test_row"].max()) + 1, int(d["raw_test_col"].max()) + 1
    (_, tidx, tval), trow, _ = ca.coo_to_csr(tm, tn, d["raw_test_row"], d["raw_test_col"],
                                             d["raw_test_val"], csc=False)
    assert np.array_equal(trow, d["R_test_coo_row"])
    assert np.array_equal(tidx, d["R_test_coo_col"])
    assert np.array_equal(tval, d["R_test_coo_data"].astype(np.float32))


@pytest.mark.parametrize("seed,rows,cols,n", [(0, 300, 200, 20000), (1, 1, 1, 50), (2, 5, 7000, 300),
                                              (3, 9000, 3, 400), (4, 10, 10, 0), (5, 2, 2, 5000),
                                              (6, 70000, 300, 250000)])
def test_gpu_builder_equals_the_oracle_and_scipy(seed, rows, cols, n):
    r, c, v = random_triples(seed, rows, cols, n)
    got = ca.coo_to_csr(rows, cols, r, c, v)
    _same(got, OC.coo_to_csr(rows, cols, r, c, v))
    sp = pytest.importorskip("scipy.sparse")
    A = sp.coo_matrix((v.astype(np.float64), (r, c)), shape=(rows, cols)).tocsr()
    assert np.array_equal(got[0][0], A.indptr) and np.array_equal(got[0][1], A.indices)
    assert np.array_equal(got[0][2], A.data.astype(np.float32))


def test_gpu_builder_on_a_workload_in_shuffled_order():
    """Scaled workload 2 (half stars, 90k ratings): its CSR shuffled into triples and rebuilt
    gives the CSR back, and the CSC equals the library's transpose."""
    tr, te, info = ca.synth_generate(2, scale=0.1)
    m, n = info["m"], info["n"]
    ptr, idx, val = tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals
    rows = np.repeat(np.arange(m, dtype=np.int32), np.diff(ptr))
    perm = np.random.default_rng(9).permutation(len(idx))
    (p, i, v), crow, (cp, ri, cv) = ca.coo_to_csr(m, n, rows[perm], idx[perm], val[perm])
    assert np.array_equal(p, ptr) and np.array_equal(i, idx) and np.array_equal(v, val)
    assert np.array_equal(crow, rows)
    wcp, wri, wcv = ca.csr_to_csc(m, n, ptr, idx, val)
    assert np.array_equal(cp, wcp) and np.array_equal(ri, wri) and np.array_equal(cv, wcv)


def test_gpu_builder_device_entry_point_and_rejections():
    import torch

    from cuda_als_gb300._lib import CsrView, lib

    r, c, v = random_triples(7, 500, 400, 30000)
    want = OC.coo_to_csr(500, 400, r, c, v)
    dev = torch.device("cuda")
    tr, tc, tv = (torch.as_tensor(a, device=dev) for a in (r, c, v))
    nz = len(v)
    out = [torch.zeros(501, dtype=torch.int32, device=dev), torch.zeros(nz, dtype=torch.int32, device=dev),
           torch.zeros(nz, dtype=torch.float32, device=dev), torch.zeros(nz, dtype=torch.int32, device=dev),
           torch.zeros(401, dtype=torch.int32, device=dev), torch.zeros(nz, dtype=torch.int32, device=dev),
           torch.zeros(nz, dtype=torch.float32, device=dev)]
    view = CsrView(500, 400, nz, C.c_void_p(tr.data_ptr()), C.c_void_p(tc.data_ptr()),
                   C.c_void_p(tv.data_ptr()))
    k = C.c_int64()
    st = torch.cuda.current_stream()
    rc = lib().als_coo_to_csr_device(C.byref(view), *[C.c_void_p(t.data_ptr()) for t in out],
                                     C.byref(k), C.c_void_p(st.cuda_stream))
    assert rc == 0
    kk = k.value
    got = ((out[0].cpu().numpy(), out[1][:kk].cpu().numpy(), out[2][:kk].cpu().numpy()),
           out[3][:kk].cpu().numpy(),
           (out[4].cpu().numpy(), out[5][:kk].cpu().numpy(), out[6][:kk].cpu().numpy()))
    _same(got, want)
    # an index out of range is an error, not a fault
    bad_c = c.copy()
    bad_c[123] = 400
    with pytest.raises(ca.ALSError) as e:
        ca.coo_to_csr(500, 400, r, bad_c, v)
    assert e.value.status == ca.Status.INVALID_ARG
    bad_r = r.copy()
    bad_r[7] = -1
    with pytest.raises(ca.ALSError):
        ca.coo_to_csr(500, 400, bad_r, c, v)
