"""GB300-native ALS sweep: the Python face of the C ABI in include/als_gb300.h.

The names mirror vserdyuk/cuda_als so its usage reads the same:

    train = host_sparse_matrix(m, n, nnz_train)          # cuda_sparse_matrix.h:8-38
    train.load_csc(...); train.load_csr(...); train.load_coo(...)
    test = host_sparse_matrix(m, n, nnz_test); test.load_coo(...)
    model = als_model(train, test, f, lambda_, iters,     # als_model.h:29-32
                      CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR, SOLVE_TYPE.LU, 32, 1, 1)
    model.train(); model.rsme_test(); model.save_libmf(path)

All compute runs in libals_gb300.so (hand-written sm_103a CUDA behind a torch-free C++ host).
"""
from __future__ import annotations

import ctypes as C
import os
from enum import IntEnum

import numpy as np

from . import _lib
from ._lib import Config, CsrView, lib

__all__ = [
    "ALSError", "CALCULATE_VTVS_TYPE", "SOLVE_TYPE", "PRECISION", "Status", "als_model",
    "host_sparse_matrix", "default_config", "config_from_ini", "csr_to_csc", "degree_order",
    "synth_generate", "synth_shape", "version", "load_dataset", "partition_rows",
    "EVENT_TYPE", "logger", "ini_get",
]


class Status(IntEnum):
    OK = 0
    INVALID_ARG = 1
    IO = 2
    CUDA = 3
    NUMERIC = 4
    TIMEOUT = 5
    UNSUPPORTED = 6
    OUT_OF_MEMORY = 7
    NO_DEVICE = 8


class CALCULATE_VTVS_TYPE(IntEnum):
    """als_model::CALCULATE_VTVS_TYPE (als_model.h:12-21)."""

    SIMPLE = 0
    SMEM_ROW_MAJOR = 1
    SMEM_COL_MAJOR = 2
    SMEM_ROW_MAJOR_NO_CALC = 3
    SMEM_COL_MAJOR_TWO_THREADS = 4
    SMEM_ROW_MAJOR_TENSOR = 5
    SMEM_ROW_MAJOR_TENSOR_SYMMETRIC = 6
    SMEM_ROW_MAJOR_TENSOR_SYMMETRIC_MULT_FRAG = 7


class SOLVE_TYPE(IntEnum):
    """als_model::SOLVE_TYPE (als_model.h:23-27) plus this build's Cholesky and autotuned."""

    LU = 0
    CUMF_ALS_CG_FP16 = 1
    CUMF_ALS_CG_FP32 = 2
    CHOLESKY = 3
    AUTO = 4


class PRECISION(IntEnum):
    FROM_VTVS = -1
    FP32 = 0
    BF16 = 1
    FP8 = 2


class ALSError(RuntimeError):
    """A non-OK als_status, with the library's message."""

    def __init__(self, status: int, message: str):
        self.status = Status(status) if status in Status._value2member_map_ else status
        super().__init__(f"{getattr(self.status, 'name', status)}: {message}")


def _check(status: int, handle=None) -> None:
    if status != 0:
        msg = lib().als_last_error(handle)
        raise ALSError(status, (msg or b"").decode(errors="replace"))


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def version() -> str:
    return lib().als_version().decode()


def default_config(**overrides) -> Config:
    cfg = Config()
    lib().als_config_default(C.byref(cfg))
    for k, v in overrides.items():
        setattr(cfg, "lambda_" if k == "lambda" else k, v)
    return cfg


def config_from_ini(path: str):
    """Parse a reference INI file -> (Config, dict of [data]/[general] values)."""
    cfg = Config()
    m, n, nt, ns = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
    runs = C.c_int32()
    folder = C.create_string_buffer(4096)
    _check(lib().als_config_from_ini(os.fsencode(path), C.byref(cfg), C.byref(m), C.byref(n),
                                     C.byref(nt), C.byref(ns), C.byref(runs), folder, 4096))
    return cfg, {"m": m.value, "n": n.value, "nnz_train": nt.value, "nnz_test": ns.value,
                 "als_runs": runs.value, "data_folder": folder.value.decode()}


def ini_get(path: str, section: str, key: str) -> str:
    """A string value of an INI file, "" when absent (INIReader::Get, main.cpp:36, :49)."""
    buf = C.create_string_buffer(4096)
    _check(lib().als_ini_get(os.fsencode(path), section.encode(), key.encode(), buf, 4096))
    return buf.value.decode()


class EVENT_TYPE(IntEnum):
    """logger::EVENT_TYPE (logger.h:8-13)."""

    ALS_UPDATE_U = 0
    ALS_UPDATE_V = 1
    ALS_ITER = 2
    MF_MODEL_TRAINING = 3


class logger:
    """Mirror of the reference's logger (logger.h:7-48) over the library's event log.

    ``logger(log_folder)`` is logger::init; ``log``, ``event_started``, ``event_finished`` and
    ``save`` keep their meaning and CSV columns; ``run_iter`` / ``als_iter`` are the columns of the
    following lines.  Attach it to a model with ``als_model.set_logger`` and ``train()`` writes the
    reference's training lines and per-iteration events into it.
    """

    def __init__(self, log_folder: str = ""):
        self._lg = C.c_void_p()
        _check(lib().als_log_create(os.fsencode(str(log_folder)), C.byref(self._lg)))
        self.log_folder = str(log_folder)

    def close(self):
        if getattr(self, "_lg", None) and self._lg.value:
            lib().als_log_destroy(self._lg)
            self._lg = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _iters(self):
        r, a = C.c_int64(), C.c_int64()
        _check(lib().als_log_get_iters(self._lg, C.byref(r), C.byref(a)))
        return r.value, a.value

    @property
    def run_iter(self) -> int:
        return self._iters()[0]

    @run_iter.setter
    def run_iter(self, v: int):
        _check(lib().als_log_set_iters(self._lg, int(v), self._iters()[1]))

    @property
    def als_iter(self) -> int:
        return self._iters()[1]

    @als_iter.setter
    def als_iter(self, v: int):
        _check(lib().als_log_set_iters(self._lg, self._iters()[0], int(v)))

    @property
    def log_name(self) -> str:
        return lib().als_log_name(self._lg).decode()

    def log(self, text: str, write_cout: bool = False):
        _check(lib().als_log_text(self._lg, text.encode(), int(bool(write_cout))))

    def event_started(self, event_type):
        _check(lib().als_log_event_started(self._lg, int(event_type)))

    def event_finished(self, event_type, write_cout: bool = False):
        _check(lib().als_log_event_finished(self._lg, int(event_type), int(bool(write_cout))))

    def text(self) -> str:
        """The CSV so far."""
        n = C.c_size_t(0)
        _check(lib().als_log_contents(self._lg, None, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        _check(lib().als_log_contents(self._lg, buf, C.byref(n)))
        return buf.value.decode()

    def save(self, log_path: str | None = None):
        """Write to log_path, or to <log_folder>/<log_name> (logger::save)."""
        _check(lib().als_log_save(self._lg, None if log_path is None else os.fsencode(str(log_path))))


class _Pinned:
    """A page-locked host buffer exposed as a numpy array (cudaMallocHost)."""

    def __init__(self, count: int, dtype):
        self.dtype = np.dtype(dtype)
        self.ptr = C.c_void_p()
        _check(lib().als_host_alloc(max(1, count) * self.dtype.itemsize, C.byref(self.ptr)))
        buf = (C.c_byte * (max(1, count) * self.dtype.itemsize)).from_address(self.ptr.value)
        self.array = np.frombuffer(buf, dtype=self.dtype, count=count)

    def __del__(self):
        try:
            if self.ptr:
                lib().als_host_free(self.ptr)
        except Exception:  # interpreter shutdown
            pass


class host_sparse_matrix:
    """Mirror of host_sparse_matrix (cuda_sparse_matrix.h:8-38): CSR, CSC and COO arrays of one
    rating matrix in host memory, loaded from the reference's raw .bin files (file size must equal
    the expected buffer size, cuda_sparse_matrix.cpp:6-27) or set from numpy arrays.  With
    pinned=True the arrays live in page-locked memory, like the reference's cudaMallocHost."""

    def __init__(self, row_cnt: int, col_cnt: int, val_cnt: int, pinned: bool = False):
        self.row_cnt, self.col_cnt, self.val_cnt = int(row_cnt), int(col_cnt), int(val_cnt)
        self.pinned = pinned
        self._keep = []
        self.has_csr = self.has_csc = self.has_coo = False
        self.h_csr_coo_vals = self.h_csr_row_ptrs = self.h_csr_coo_col_idxs = None
        self.h_coo_row_idxs = None
        self.h_csc_vals = self.h_csc_row_idxs = self.h_csc_col_ptrs = None

    def _buffer(self, count, dtype):
        if self.pinned:
            b = _Pinned(count, dtype)
            self._keep.append(b)
            return b.array
        return np.empty(count, dtype=dtype)

    def _load(self, path, count, dtype):
        a = self._buffer(count, dtype)
        _check(lib().als_load_bin(os.fsencode(str(path)), _ptr(a), a.nbytes))
        return a

    def _own(self, a, dtype):
        a = np.asarray(a, dtype=dtype).ravel()
        if not self.pinned:
            return np.ascontiguousarray(a)
        b = self._buffer(a.size, dtype)
        b[:] = a
        return b

    # cuda_sparse_matrix.cpp:43-51 / 53-59 / 61-69 (CSR and COO share vals and col_idxs)
    def load_csr(self, vals_path, row_ptrs_path, col_idxs_path):
        if not self.has_coo:
            self.h_csr_coo_vals = self._load(vals_path, self.val_cnt, np.float32)
            self.h_csr_coo_col_idxs = self._load(col_idxs_path, self.val_cnt, np.int32)
        self.h_csr_row_ptrs = self._load(row_ptrs_path, self.row_cnt + 1, np.int32)
        self.has_csr = True

    def load_csc(self, vals_path, row_idxs_path, col_ptrs_path):
        self.h_csc_vals = self._load(vals_path, self.val_cnt, np.float32)
        self.h_csc_row_idxs = self._load(row_idxs_path, self.val_cnt, np.int32)
        self.h_csc_col_ptrs = self._load(col_ptrs_path, self.col_cnt + 1, np.int32)
        self.has_csc = True

    def load_coo(self, vals_path, row_idxs_path, col_idxs_path):
        if not self.has_csr:
            self.h_csr_coo_vals = self._load(vals_path, self.val_cnt, np.float32)
            self.h_csr_coo_col_idxs = self._load(col_idxs_path, self.val_cnt, np.int32)
        self.h_coo_row_idxs = self._load(row_idxs_path, self.val_cnt, np.int32)
        self.has_coo = True

    def set_csr(self, row_ptrs, col_idxs, vals):
        self.h_csr_row_ptrs = self._own(row_ptrs, np.int32)
        self.h_csr_coo_col_idxs = self._own(col_idxs, np.int32)
        self.h_csr_coo_vals = self._own(vals, np.float32)
        self.has_csr = True
        return self

    def set_csc(self, col_ptrs, row_idxs, vals):
        self.h_csc_col_ptrs = self._own(col_ptrs, np.int32)
        self.h_csc_row_idxs = self._own(row_idxs, np.int32)
        self.h_csc_vals = self._own(vals, np.float32)
        self.has_csc = True
        return self

    def set_coo(self, row_idxs, col_idxs, vals):
        self.h_coo_row_idxs = self._own(row_idxs, np.int32)
        if not self.has_csr:
            self.h_csr_coo_col_idxs = self._own(col_idxs, np.int32)
            self.h_csr_coo_vals = self._own(vals, np.float32)
        self.has_coo = True
        return self

    def csr_view(self) -> CsrView:
        if not self.has_csr:
            raise ALSError(Status.INVALID_ARG, "matrix has no CSR arrays")
        return CsrView(self.row_cnt, self.col_cnt, self.val_cnt, _ptr(self.h_csr_row_ptrs),
                       _ptr(self.h_csr_coo_col_idxs), _ptr(self.h_csr_coo_vals))

    def csc_view(self):
        if not self.has_csc:
            return None
        return CsrView(self.row_cnt, self.col_cnt, self.val_cnt, _ptr(self.h_csc_col_ptrs),
                       _ptr(self.h_csc_row_idxs), _ptr(self.h_csc_vals))

    def coo_view(self):
        if not self.has_coo:
            return None
        return CsrView(self.row_cnt, self.col_cnt, self.val_cnt, _ptr(self.h_coo_row_idxs),
                       _ptr(self.h_csr_coo_col_idxs), _ptr(self.h_csr_coo_vals))


def load_dataset(data_folder: str, m: int, n: int, nnz_train: int, nnz_test: int,
                 pinned: bool = False):
    """The loads of main.cpp:68-75: train CSC + CSR + COO rows, test COO, same file names."""
    d = str(data_folder)
    tr = host_sparse_matrix(m, n, nnz_train, pinned)
    tr.load_csc(f"{d}/R_train_csc.data.bin", f"{d}/R_train_csc.indices.bin",
                f"{d}/R_train_csc.indptr.bin")
    tr.load_csr(f"{d}/R_train_csr.data.bin", f"{d}/R_train_csr.indptr.bin",
                f"{d}/R_train_csr.indices.bin")
    tr.load_coo(f"{d}/R_train_csr.data.bin", f"{d}/R_train_coo.row.bin",
                f"{d}/R_train_csr.indices.bin")
    te = host_sparse_matrix(m, n, nnz_test, pinned)
    te.load_coo(f"{d}/R_test_coo.data.bin", f"{d}/R_test_coo.row.bin",
                f"{d}/R_test_coo.col.bin")
    return tr, te


class als_model:
    """Mirror of als_model (als_model.h:11-80) over the C ABI.

    The constructor copies the training CSR (+ CSC when the matrix carries one; otherwise the CSC
    is built by the GPU transpose) and the test COO to the device.  ``train()`` re-initialises the
    factors with the reference's srand(0) scheme, runs ``iters`` iterations and copies the factors
    into ``h_UT`` / ``h_VT``.  Keyword options set the [als_gb300] fields of als_config
    (precision, refine_steps, cond_threshold, cg_steps, cg_tol, use_graph, autotune, device).
    """

    def __init__(self, host_train_ratings: host_sparse_matrix,
                 host_test_ratings: host_sparse_matrix | None, f: int, lambda_: float,
                 iters: int, calculate_vtvs_type=CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR,
                 solve_type=SOLVE_TYPE.LU, smem_col_cnt: int = 32, m_batches: int = 1,
                 n_batches: int = 1, device_views: bool = False, **options):
        cfg = default_config()
        cfg.f, cfg.lambda_, cfg.iters = int(f), float(lambda_), int(iters)
        cfg.calculate_vtvs_type, cfg.solve_type = int(calculate_vtvs_type), int(solve_type)
        cfg.smem_col_cnt, cfg.m_batches, cfg.n_batches = smem_col_cnt, m_batches, n_batches
        for k, v in options.items():
            if not hasattr(cfg, k):
                raise TypeError(f"unknown option {k}")
            setattr(cfg, k, v)
        self.config = cfg
        self.m, self.n, self.f = host_train_ratings.row_cnt, host_train_ratings.col_cnt, int(f)
        self.lambda_, self.iters = float(lambda_), int(iters)
        self.calculate_vtvs_type, self.solve_type = calculate_vtvs_type, solve_type
        self.smem_col_cnt, self.m_batches, self.n_batches = smem_col_cnt, m_batches, n_batches
        csr = host_train_ratings.csr_view()
        csc = host_train_ratings.csc_view()
        coo = host_test_ratings.coo_view() if host_test_ratings is not None else None
        self._h = C.c_void_p()
        create = lib().als_create_device if device_views else lib().als_create
        _check(create(C.byref(cfg), C.byref(csr), C.byref(csc) if csc is not None else None,
                      C.byref(coo) if coo is not None else None, C.byref(self._h)))
        self.h_UT = np.zeros((self.m, self.f), np.float32)
        self.h_VT = np.zeros((self.n, self.f), np.float32)

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().als_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _c(self, status):
        _check(status, self._h)

    # -- the reference's methods
    def train(self):
        self._c(lib().als_train(self._h))
        self.get_factors(self.h_UT, self.h_VT)

    def rsme_train(self) -> float:
        out = C.c_double()
        self._c(lib().als_rmse_train(self._h, C.byref(out)))
        return out.value

    def rsme_test(self) -> float:
        out = C.c_double()
        self._c(lib().als_rmse_test(self._h, C.byref(out)))
        return out.value

    def save_libmf(self, path: str):
        self._c(lib().als_save_libmf(self._h, os.fsencode(str(path))))

    # -- extensions
    def init_factors(self):
        self._c(lib().als_init_factors(self._h))

    def iterate(self, iters: int = 1):
        self._c(lib().als_iterate(self._h, int(iters)))

    def set_logger(self, lg: "logger | None", iter_rmse: bool = False, write_cout: bool = False):
        """Attach an event log: train() / iterate() then write the reference's training lines,
        per-iteration ALS_UPDATE_U / ALS_UPDATE_V / ALS_ITER events and, with iter_rmse, the test
        RMSE after every iteration but the last.  None detaches."""
        self._logger = lg
        self._c(lib().als_set_log(self._h, None if lg is None else lg._lg, int(bool(iter_rmse)),
                                  int(bool(write_cout))))

    def half_sweep(self, side: int):
        """side 0 solves U given V (the U block of train), side 1 solves V given U."""
        self._c(lib().als_half_sweep(self._h, int(side)))

    def reload(self, host_train_ratings: host_sparse_matrix,
               host_test_ratings: host_sparse_matrix | None = None):
        """Upload a new rating snapshot of the same sizes (als_reload); factors are kept."""
        csr = host_train_ratings.csr_view()
        csc = host_train_ratings.csc_view()
        coo = host_test_ratings.coo_view() if host_test_ratings is not None else None
        self._c(lib().als_reload(self._h, C.byref(csr), C.byref(csc) if csc is not None else None,
                                 C.byref(coo) if coo is not None else None))

    def update_values(self, csr_vals):
        a = np.ascontiguousarray(csr_vals, dtype=np.float32)
        self._c(lib().als_update_values(self._h, _ptr(a)))

    def get_factors(self, U=None, V=None):
        U = np.empty((self.m, self.f), np.float32) if U is None else U
        V = np.empty((self.n, self.f), np.float32) if V is None else V
        self._c(lib().als_get_factors(self._h, _ptr(U), _ptr(V)))
        return U, V

    def set_factors(self, U=None, V=None):
        U = None if U is None else np.ascontiguousarray(U, dtype=np.float32)
        V = None if V is None else np.ascontiguousarray(V, dtype=np.float32)
        self._c(lib().als_set_factors(self._h, _ptr(U), _ptr(V)))

    def device_factors(self):
        u, v = C.c_void_p(), C.c_void_p()
        self._c(lib().als_get_device_factors(self._h, C.byref(u), C.byref(v)))
        return u.value, v.value

    def set_stream(self, stream_ptr: int | None):
        self._c(lib().als_set_stream(self._h, stream_ptr))

    def set_wait_limit_ns(self, ns: int = 0):
        """Bound of the sweep kernels' device waits in ns (0: the default, 10 s)."""
        self._c(lib().als_set_wait_limit_ns(self._h, int(ns)))

    def stage_ms(self):
        out = (C.c_double * 4)()
        self._c(lib().als_get_stage_ms(self._h, out))
        return {"U": out[0], "V": out[1], "quantise": out[2], "transpose": out[3]}

    def counters(self):
        out = (C.c_int64 * 3)()
        self._c(lib().als_get_counters(self._h, out))
        return {"launches": out[0], "flagged_rows": out[1], "fp64_refined_rows": out[2]}

    def plan(self, side: int):
        nb = C.c_int32(64)
        lo, kind, solver = (np.zeros(64, np.int32) for _ in range(3))
        self._c(lib().als_get_plan(self._h, side, _ptr(lo), _ptr(kind), _ptr(solver),
                                   C.byref(nb)))
        k = nb.value
        return [{"lo": int(lo[i]), "kind": int(kind[i]), "solver": int(solver[i])}
                for i in range(k)]

    def tuning(self, side: int):
        """The autotuner's per-bucket measurements (ALS_SOLVE_AUTO): FP32-CG, Cholesky and (tensor-
        core precisions) FP16-Gram-CG ms on the tuning sweep and each CG's relative difference to
        the Cholesky solution; negative = not measured; [] when nothing was tuned."""
        nb = C.c_int32(64)
        cg, ch, rel, cg16, rel16 = (np.zeros(64, np.float32) for _ in range(5))
        self._c(lib().als_get_tuning(self._h, side, _ptr(cg), _ptr(ch), _ptr(rel), _ptr(cg16),
                                     _ptr(rel16), C.byref(nb)))
        return [{"ms_cg": float(cg[i]), "ms_cholesky": float(ch[i]), "rel_diff": float(rel[i]),
                 "ms_cg16": float(cg16[i]), "rel_diff_cg16": float(rel16[i])}
                for i in range(nb.value)]

    def user_halfsweep_adjoint(self, rows, cols, vals):
        """Held-out loss of the user half-sweep, dL/dV (n x f) and dL/dlambda."""
        rows = np.ascontiguousarray(rows, np.int32)
        cols = np.ascontiguousarray(cols, np.int32)
        vals = np.ascontiguousarray(vals, np.float32)
        view = CsrView(self.m, self.n, len(vals), _ptr(rows), _ptr(cols), _ptr(vals))
        loss, dlam = C.c_double(), C.c_double()
        G = np.zeros((self.n, self.f), np.float32)
        self._c(lib().als_user_halfsweep_adjoint(self._h, C.byref(view), C.byref(loss), _ptr(G),
                                                 C.byref(dlam)))
        return loss.value, G, dlam.value

    def user_halfsweep_adjoint_f64(self, rows, cols, vals, Y, lambda_: float):
        """The same in FP64 on the GPU from FP64 item factors Y (n x f) and lambda:
        (loss, dL/dY as float64 n x f, dL/dlambda)."""
        rows = np.ascontiguousarray(rows, np.int32)
        cols = np.ascontiguousarray(cols, np.int32)
        vals = np.ascontiguousarray(vals, np.float32)
        Y = np.ascontiguousarray(Y, np.float64)
        view = CsrView(self.m, self.n, len(vals), _ptr(rows), _ptr(cols), _ptr(vals))
        loss, dlam = C.c_double(), C.c_double()
        G = np.zeros((self.n, self.f), np.float64)
        self._c(lib().als_user_halfsweep_adjoint_f64(self._h, C.byref(view), _ptr(Y),
                                                     float(lambda_), C.byref(loss), _ptr(G),
                                                     C.byref(dlam)))
        return loss.value, G, dlam.value


# ------------------------------------------------------------------------------------------------
# standalone index kernels and the synthetic workloads


def csr_to_csc(rows: int, cols: int, row_ptrs, col_idxs, vals):
    """Stable GPU transpose (scipy tocsc order) -> (col_ptrs, row_idxs, vals)."""
    p = np.ascontiguousarray(row_ptrs, np.int32)
    i = np.ascontiguousarray(col_idxs, np.int32)
    v = np.ascontiguousarray(vals, np.float32)
    view = CsrView(rows, cols, len(i), _ptr(p), _ptr(i), _ptr(v))
    cp = np.zeros(cols + 1, np.int32)
    ri = np.zeros(len(i), np.int32)
    cv = np.zeros(len(i), np.float32)
    _check(lib().als_csr_to_csc(C.byref(view), _ptr(cp), _ptr(ri), _ptr(cv)))
    return cp, ri, cv


def coo_to_csr(rows: int, cols: int, row_idxs, col_idxs, vals, csc: bool = True):
    """Rating triples -> (CSR (row_ptrs, col_idxs, vals), the row of each CSR entry, and the CSC
    (col_ptrs, row_idxs, vals) or None), built on the GPU: scipy's coo_matrix(...).tocsr() /
    .tocoo() / .tocsc() order, duplicates summed (FP64, rounded once to FP32)."""
    r = np.ascontiguousarray(row_idxs, np.int32)
    c = np.ascontiguousarray(col_idxs, np.int32)
    v = np.ascontiguousarray(vals, np.float32)
    view = CsrView(rows, cols, len(v), _ptr(r), _ptr(c), _ptr(v))
    nz = len(v)
    ptr = np.zeros(rows + 1, np.int32)
    idx, val, crow = np.zeros(nz, np.int32), np.zeros(nz, np.float32), np.zeros(nz, np.int32)
    cptr = np.zeros(cols + 1, np.int32) if csc else None
    ridx = np.zeros(nz, np.int32) if csc else None
    cval = np.zeros(nz, np.float32) if csc else None
    out = C.c_int64()
    _check(lib().als_coo_to_csr(C.byref(view), _ptr(ptr), _ptr(idx), _ptr(val), _ptr(crow),
                                _ptr(cptr), _ptr(ridx), _ptr(cval), C.byref(out)))
    k = out.value
    return ((ptr, idx[:k], val[:k]), crow[:k],
            (cptr, ridx[:k], cval[:k]) if csc else None)


def degree_order(row_ptrs):
    p = np.ascontiguousarray(row_ptrs, np.int32)
    perm = np.zeros(len(p) - 1, np.int32)
    _check(lib().als_degree_order(len(p) - 1, _ptr(p), _ptr(perm)))
    return perm


def partition_rows(row_ptrs, nparts: int, row_weight: float = 0.0):
    """Contiguous, weight-balanced row ranges for nparts ranks -> bounds (nparts + 1 int64)."""
    p = np.ascontiguousarray(row_ptrs, np.int32)
    bounds = np.zeros(nparts + 1, np.int64)
    _check(lib().als_partition_rows(len(p) - 1, _ptr(p), int(nparts), float(row_weight),
                                    _ptr(bounds)))
    return bounds


def synth_shape(config: int):
    m, n, nnz, f, lam = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int32(), C.c_float()
    _check(lib().als_synth_shape(config, C.byref(m), C.byref(n), C.byref(nnz), C.byref(f),
                                 C.byref(lam)))
    return {"m": m.value, "n": n.value, "nnz": nnz.value, "f": f.value, "lambda": lam.value}


def synth_generate(config: int, seed: int | None = None, scale: float = 1.0,
                   pinned: bool = False):
    """Seeded synthetic workload (see synth.cpp) -> (train host_sparse_matrix with CSR,
    test host_sparse_matrix with COO, info dict).  Default seed 0xA15 + config (config 4:
    0xA15 + 3)."""
    # config 4 is config 3 transposed, so it shares config 3's default seed
    seed = 0xA15 + (3 if config == 4 else config) if seed is None else seed
    m, n, nt, ns = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
    L = lib()
    _check(L.als_synth_generate(config, seed, scale, C.byref(m), C.byref(n), C.byref(nt),
                                C.byref(ns), None, None, None, None, None, None))
    tr = host_sparse_matrix(m.value, n.value, nt.value, pinned)
    te = host_sparse_matrix(m.value, n.value, ns.value, pinned)
    ptr = tr._buffer(m.value + 1, np.int32)
    col = tr._buffer(nt.value, np.int32)
    val = tr._buffer(nt.value, np.float32)
    trow = te._buffer(ns.value, np.int32)
    tcol = te._buffer(ns.value, np.int32)
    tval = te._buffer(ns.value, np.float32)
    _check(L.als_synth_generate(config, seed, scale, C.byref(m), C.byref(n), C.byref(nt),
                                C.byref(ns), _ptr(ptr), _ptr(col), _ptr(val), _ptr(trow),
                                _ptr(tcol), _ptr(tval)))
    tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals = ptr, col, val
    tr.has_csr = True
    te.h_coo_row_idxs, te.h_csr_coo_col_idxs, te.h_csr_coo_vals = trow, tcol, tval
    te.has_coo = True
    shp = synth_shape(config)
    info = {"config": config, "seed": seed, "scale": scale, "m": m.value, "n": n.value,
            "nnz_train": nt.value, "nnz_test": ns.value, "f": shp["f"], "lambda": shp["lambda"]}
    return tr, te, info
