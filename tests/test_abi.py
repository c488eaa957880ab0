"""The C ABI boundary without a GPU: exports, struct layout, defaults, INI keys, .bin loaders,
synthetic workloads, and loud failure when no device is present (CPU only)."""
from __future__ import annotations

import ctypes as C
import re

import numpy as np
import pytest

import cuda_als_gb300 as ca
from cuda_als_gb300 import _lib
from conftest import ROOT, load_toy

HEADER = ROOT / "include" / "als_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^[a-z][\w \*]*?\b(als_\w+)\(", text, re.M)))


def test_every_declared_symbol_is_exported():
    names = declared_functions()
    assert len(names) >= 30
    L = C.CDLL(str(_lib.LIB_PATH))
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert sorted(_lib.EXPORTS) == names


def test_config_struct_layout_and_defaults():
    assert C.sizeof(_lib.Config) == 16 * 4
    cfg = ca.default_config()
    assert (cfg.f, cfg.iters, cfg.calculate_vtvs_type, cfg.solve_type, cfg.smem_col_cnt) == (
        100, 10, 1, 0, 32)
    assert cfg.lambda_ == pytest.approx(0.05)
    assert (cfg.cg_steps, cfg.precision) == (6, ca.PRECISION.FROM_VTVS)
    assert cfg.cg_tol == pytest.approx(1e-4)


INI = """\
[general]
log_folder = log/example
; multiple runs
als_runs = 3

[data]
data_folder = data/example
m = 1234
n = 567
nnz_train = 8900
nnz_test = 100

[als]
f = 64
lambda = 0.048
als_iters = 7
als_calculate_vtvs_type = 6
als_solve_type = 2
m_batches = 4
n_batches = 2

[als_gb300]
precision = bf16
cg_steps = 3
refine_steps = 2
"""


def test_ini_keys_of_the_reference(tmp_path):
    p = tmp_path / "x.ini"
    p.write_text(INI)
    cfg, d = ca.config_from_ini(str(p))
    assert d == {"m": 1234, "n": 567, "nnz_train": 8900, "nnz_test": 100, "als_runs": 3,
                 "data_folder": "data/example"}
    assert (cfg.f, cfg.iters, cfg.calculate_vtvs_type, cfg.solve_type) == (64, 7, 6, 2)
    assert (cfg.m_batches, cfg.n_batches, cfg.smem_col_cnt) == (4, 2, 32)
    assert cfg.lambda_ == pytest.approx(0.048)
    assert (cfg.precision, cfg.cg_steps, cfg.refine_steps) == (ca.PRECISION.BF16, 3, 2)


def test_ini_missing_file_is_io_error():
    with pytest.raises(ca.ALSError) as e:
        ca.config_from_ini("/nonexistent/x.ini")
    assert e.value.status == ca.Status.IO


def _write_dataset(tmp_path, t):
    d = tmp_path
    (t["R_train_csr_data"].astype(np.float32)).tofile(d / "R_train_csr.data.bin")
    t["R_train_csr_indptr"].astype(np.int32).tofile(d / "R_train_csr.indptr.bin")
    t["R_train_csr_indices"].astype(np.int32).tofile(d / "R_train_csr.indices.bin")
    t["R_train_csc_data"].astype(np.float32).tofile(d / "R_train_csc.data.bin")
    t["R_train_csc_indptr"].astype(np.int32).tofile(d / "R_train_csc.indptr.bin")
    t["R_train_csc_indices"].astype(np.int32).tofile(d / "R_train_csc.indices.bin")
    np.repeat(np.arange(t["m"]), np.diff(t["R_train_csr_indptr"])).astype(np.int32).tofile(
        d / "R_train_coo.row.bin")
    t["R_test_coo_data"].astype(np.float32).tofile(d / "R_test_coo.data.bin")
    t["R_test_coo_row"].astype(np.int32).tofile(d / "R_test_coo.row.bin")
    t["R_test_coo_col"].astype(np.int32).tofile(d / "R_test_coo.col.bin")


@pytest.mark.parametrize("pinned", [False])
def test_loaders_read_the_reference_file_set(tmp_path, toy, pinned):
    _write_dataset(tmp_path, toy)
    nnz, nt = len(toy["R_train_csr_data"]), len(toy["R_test_coo_data"])
    tr, te = ca.load_dataset(str(tmp_path), toy["m"], toy["n"], nnz, nt, pinned=pinned)
    assert tr.has_csr and tr.has_csc and tr.has_coo and te.has_coo
    assert np.array_equal(tr.h_csr_row_ptrs, toy["R_train_csr_indptr"])
    assert np.array_equal(tr.h_csc_row_idxs, toy["R_train_csc_indices"])
    assert np.array_equal(te.h_coo_row_idxs, toy["R_test_coo_row"])
    assert np.array_equal(te.h_csr_coo_vals, toy["R_test_coo_data"].astype(np.float32))


def test_loader_rejects_wrong_size(tmp_path):
    np.zeros(10, np.float32).tofile(tmp_path / "a.bin")
    m = ca.host_sparse_matrix(3, 3, 11)
    with pytest.raises(ca.ALSError) as e:
        m.load_coo(str(tmp_path / "a.bin"), str(tmp_path / "a.bin"), str(tmp_path / "a.bin"))
    assert e.value.status == ca.Status.IO
    with pytest.raises(ca.ALSError):
        m.load_csc(str(tmp_path / "missing.bin"), "", "")


def _no_device() -> bool:
    try:
        import torch

        return not torch.cuda.is_available()
    except Exception:
        return True


@pytest.mark.skipif(not _no_device(), reason="a GPU is visible")
def test_no_device_fails_loudly():
    t = load_toy("toy_data_2")
    tr = ca.host_sparse_matrix(t["m"], t["n"], len(t["R_train_csr_data"])).set_csr(
        t["R_train_csr_indptr"], t["R_train_csr_indices"], t["R_train_csr_data"])
    with pytest.raises(ca.ALSError) as e:
        ca.als_model(tr, None, 8, 0.05, 1)
    assert e.value.status == ca.Status.NO_DEVICE
    with pytest.raises(ca.ALSError):
        ca.csr_to_csc(t["m"], t["n"], t["R_train_csr_indptr"], t["R_train_csr_indices"],
                      t["R_train_csr_data"])


def test_fp8_precision_is_validated_before_any_device_work(toy):
    """FP8 (e4m3) runs on the tensor-core path, f in 1..128: beyond it the configuration is
    rejected as UNSUPPORTED before any device work; within it, validation passes and (on a
    machine without a GPU) the call stops at the missing device, never at another precision."""
    tr = ca.host_sparse_matrix(toy["m"], toy["n"], len(toy["R_train_csr_data"])).set_csr(
        toy["R_train_csr_indptr"], toy["R_train_csr_indices"], toy["R_train_csr_data"])
    with pytest.raises(ca.ALSError) as e:
        ca.als_model(tr, None, 200, 0.05, 1, precision=int(ca.PRECISION.FP8))
    assert e.value.status == ca.Status.UNSUPPORTED
    with pytest.raises(ca.ALSError) as e:
        ca.als_model(tr, None, 8, 0.05, 1, precision=int(ca.PRECISION.FP8))
    assert e.value.status == ca.Status.NO_DEVICE


@pytest.mark.parametrize("config,scale", [(1, 1.0), (2, 0.05), (3, 0.03), (4, 0.03), (5, 0.03)])
def test_synthetic_workload_invariants(config, scale):
    tr, te, info = ca.synth_generate(config, scale=scale)
    m, n = info["m"], info["n"]
    ptr, col, val = tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals
    assert ptr[0] == 0 and ptr[-1] == len(col) == info["nnz_train"]
    assert np.all(np.diff(ptr) >= 1)                                # every row has a rating
    assert np.all(np.bincount(col, minlength=n) >= 1)               # every column too
    key = np.repeat(np.arange(m, dtype=np.int64), np.diff(ptr)) * n + col
    assert np.all(np.diff(key) > 0)                                 # sorted, unique
    tkey = te.h_coo_row_idxs.astype(np.int64) * n + te.h_csr_coo_col_idxs
    assert np.all(np.diff(tkey) > 0)
    assert not np.intersect1d(key, tkey).size                       # disjoint split
    allowed = np.arange(1, 6) if config in (1, 3, 4) else np.arange(1, 11) / 2
    assert np.isin(val, allowed).all()
    again = ca.synth_generate(config, scale=scale)[0]
    assert np.array_equal(again.h_csr_coo_vals, val)                # deterministic


def test_full_config_shapes():
    assert ca.synth_shape(3) == {"m": 480189, "n": 17770, "nnz": 100000000, "f": 100,
                                 "lambda": pytest.approx(0.048)}
    assert ca.synth_shape(4)["m"] == 17770 and ca.synth_shape(4)["f"] == 128
    with pytest.raises(ca.ALSError):
        ca.synth_shape(9)
