"""ctypes binding of libals_gb300.so (the C ABI declared in include/als_gb300.h).

The shared object is built in-tree by cuda_als_gb300.build.build().  There is no fallback: when
the library is missing every call raises, so a run can never silently skip the CUDA path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libals_gb300.so"

i32, i64, u64, f32, f64 = C.c_int32, C.c_int64, C.c_uint64, C.c_float, C.c_double
P = C.c_void_p
SZ = C.c_size_t


class Config(C.Structure):
    """struct als_config (include/als_gb300.h)."""

    _fields_ = [
        ("f", i32), ("lambda_", f32), ("iters", i32), ("calculate_vtvs_type", i32),
        ("solve_type", i32), ("smem_col_cnt", i32), ("m_batches", i32), ("n_batches", i32),
        ("precision", i32), ("refine_steps", i32), ("cond_threshold", f32), ("cg_steps", i32),
        ("cg_tol", f32), ("use_graph", i32), ("autotune", i32), ("device", i32),
    ]


class CsrView(C.Structure):
    _fields_ = [("rows", i64), ("cols", i64), ("nnz", i64), ("ptrs", P), ("idxs", P),
                ("vals", P)]


CscView = CsrView
CooView = CsrView  # rows, cols, nnz, row_idxs, col_idxs, vals: same memory layout

_lib = None


def lib() -> C.CDLL:
    """Load libals_gb300.so; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; "
            "g.build()'` (or cuda_als_gb300.build.build()); there is no CPU fallback")
    L = C.CDLL(str(LIB_PATH))
    H = P  # als_handle*
    sigs = {
        "als_version": ([], C.c_char_p),
        "als_status_string": ([i32], C.c_char_p),
        "als_config_default": ([C.POINTER(Config)], None),
        "als_config_from_ini": ([C.c_char_p, C.POINTER(Config), C.POINTER(i64), C.POINTER(i64),
                                 C.POINTER(i64), C.POINTER(i64), C.POINTER(i32), C.c_char_p, SZ],
                                i32),
        "als_host_alloc": ([SZ, C.POINTER(P)], i32),
        "als_host_free": ([P], i32),
        "als_load_bin": ([C.c_char_p, P, SZ], i32),
        "als_create": ([C.POINTER(Config), C.POINTER(CsrView), C.POINTER(CscView),
                        C.POINTER(CooView), C.POINTER(H)], i32),
        "als_create_device": ([C.POINTER(Config), C.POINTER(CsrView), C.POINTER(CscView),
                               C.POINTER(CooView), C.POINTER(H)], i32),
        "als_destroy": ([H], i32),
        "als_last_error": ([H], C.c_char_p),
        "als_set_stream": ([H, P], i32),
        "als_update_values": ([H, P], i32),
        "als_reload": ([H, C.POINTER(CsrView), C.POINTER(CscView), C.POINTER(CooView)], i32),
        "als_init_factors": ([H], i32),
        "als_iterate": ([H, i32], i32),
        "als_half_sweep": ([H, i32], i32),
        "als_train": ([H], i32),
        "als_rmse_test": ([H, C.POINTER(f64)], i32),
        "als_rmse_train": ([H, C.POINTER(f64)], i32),
        "als_get_factors": ([H, P, P], i32),
        "als_set_factors": ([H, P, P], i32),
        "als_get_device_factors": ([H, C.POINTER(P), C.POINTER(P)], i32),
        "als_save_libmf": ([H, C.c_char_p], i32),
        "als_get_shape": ([H, C.POINTER(i64), C.POINTER(i64), C.POINTER(i32), C.POINTER(i64),
                           C.POINTER(i64)], i32),
        "als_get_stage_ms": ([H, C.POINTER(f64)], i32),
        "als_get_counters": ([H, C.POINTER(i64)], i32),
        "als_get_plan": ([H, i32, P, P, P, C.POINTER(i32)], i32),
        "als_set_wait_limit_ns": ([H, u64], i32),
        "als_get_tuning": ([H, i32, P, P, P, P, P, C.POINTER(i32)], i32),
        "als_user_halfsweep_adjoint": ([H, C.POINTER(CooView), C.POINTER(f64), P,
                                        C.POINTER(f64)], i32),
        "als_user_halfsweep_adjoint_f64": ([H, C.POINTER(CooView), P, f64, C.POINTER(f64), P,
                                            C.POINTER(f64)], i32),
        "als_csr_to_csc": ([C.POINTER(CsrView), P, P, P], i32),
        "als_csr_to_csc_device": ([C.POINTER(CsrView), P, P, P, P], i32),
        "als_csr_to_csc_device_noalloc": ([C.POINTER(CsrView), P, P, P, P], i32),
        "als_coo_to_csr": ([C.POINTER(CooView), P, P, P, P, P, P, P, C.POINTER(i64)], i32),
        "als_coo_to_csr_device": ([C.POINTER(CooView), P, P, P, P, P, P, P, C.POINTER(i64), P],
                                  i32),
        "als_degree_order": ([i64, P, P], i32),
        "als_partition_rows": ([i64, P, i32, f64, P], i32),
        "als_log_create": ([C.c_char_p, C.POINTER(P)], i32),
        "als_log_destroy": ([P], i32),
        "als_log_text": ([P, C.c_char_p, i32], i32),
        "als_log_event_started": ([P, i32], i32),
        "als_log_event_finished": ([P, i32, i32], i32),
        "als_log_set_iters": ([P, i64, i64], i32),
        "als_log_get_iters": ([P, C.POINTER(i64), C.POINTER(i64)], i32),
        "als_log_name": ([P], C.c_char_p),
        "als_log_contents": ([P, C.c_char_p, C.POINTER(SZ)], i32),
        "als_log_save": ([P, C.c_char_p], i32),
        "als_set_log": ([H, P, i32, i32], i32),
        "als_ini_get": ([C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, SZ], i32),
        "als_synth_shape": ([i32, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64),
                             C.POINTER(i32), C.POINTER(f32)], i32),
        "als_synth_generate": ([i32, u64, f64, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64),
                                C.POINTER(i64), P, P, P, P, P, P], i32),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


# names every build of the library must export (checked by the CPU test suite)
EXPORTS = [
    "als_version", "als_status_string", "als_config_default", "als_config_from_ini",
    "als_host_alloc", "als_host_free", "als_load_bin", "als_create", "als_create_device",
    "als_destroy", "als_last_error", "als_set_stream", "als_update_values", "als_reload", "als_init_factors",
    "als_iterate", "als_half_sweep", "als_train", "als_rmse_test", "als_rmse_train",
    "als_get_factors", "als_set_factors", "als_get_device_factors", "als_save_libmf",
    "als_get_shape", "als_get_stage_ms", "als_get_counters", "als_get_plan", "als_get_tuning", "als_set_wait_limit_ns",
    "als_user_halfsweep_adjoint", "als_user_halfsweep_adjoint_f64", "als_csr_to_csc", "als_csr_to_csc_device",
    "als_csr_to_csc_device_noalloc", "als_coo_to_csr", "als_coo_to_csr_device",
    "als_degree_order", "als_partition_rows", "als_synth_shape", "als_synth_generate",
    "als_log_create", "als_log_destroy", "als_log_text", "als_log_event_started",
    "als_log_event_finished", "als_log_set_iters", "als_log_get_iters", "als_log_name",
    "als_log_contents", "als_log_save", "als_set_log", "als_ini_get",
]
