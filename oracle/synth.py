"""The seeded synthetic workloads, generated without the product library.  TEST INFRASTRUCTURE.

Loads oracle/_build/libsynth (the library's own generator source, synth.cpp, built on its own by
oracle/build.py build_synth), so that bench.py's CPU reference arm makes the same bytes as the
GPU arm while loading nothing but oracle-side code.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(str(_build.build_synth()))
        i32, i64, u64, f32, f64, P = C.c_int32, C.c_int64, C.c_uint64, C.c_float, C.c_double, C.c_void_p
        L.als_synth_shape.argtypes = [i32, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64),
                                      C.POINTER(i32), C.POINTER(f32)]
        L.als_synth_shape.restype = i32
        L.als_synth_generate.argtypes = [i32, u64, f64, C.POINTER(i64), C.POINTER(i64),
                                         C.POINTER(i64), C.POINTER(i64), P, P, P, P, P, P]
        L.als_synth_generate.restype = i32
        L.oracle_synth_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def _check(status):
    if status != 0:
        raise RuntimeError(f"synthetic generator failed ({status}): "
                           f"{lib().oracle_synth_last_error().decode()}")


def default_seed(config: int) -> int:
    """0xA15 + config; workload 4 (workload 3 transposed) shares workload 3's seed."""
    return 0xA15 + (3 if config == 4 else config)


def generate(config: int, seed: int | None = None, scale: float = 1.0):
    """-> (csr (ptr, idx, val), test COO (rows, cols, vals), info), the bytes the library's
    als_synth_generate makes for the same (config, seed, scale)."""
    seed = default_seed(config) if seed is None else seed
    L = lib()
    m, n, nt, ns = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
    _check(L.als_synth_generate(config, seed, scale, C.byref(m), C.byref(n), C.byref(nt),
                                C.byref(ns), None, None, None, None, None, None))
    ptr = np.empty(m.value + 1, np.int32)
    idx = np.empty(nt.value, np.int32)
    val = np.empty(nt.value, np.float32)
    trow = np.empty(ns.value, np.int32)
    tcol = np.empty(ns.value, np.int32)
    tval = np.empty(ns.value, np.float32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    _check(L.als_synth_generate(config, seed, scale, C.byref(m), C.byref(n), C.byref(nt),
                                C.byref(ns), p(ptr), p(idx), p(val), p(trow), p(tcol), p(tval)))
    mm, nn, nz, f, lam = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int32(), C.c_float()
    _check(L.als_synth_shape(config, C.byref(mm), C.byref(nn), C.byref(nz), C.byref(f),
                             C.byref(lam)))
    info = {"config": config, "seed": seed, "scale": scale, "m": m.value, "n": n.value,
            "nnz_train": nt.value, "nnz_test": ns.value, "f": f.value, "lambda": lam.value}
    return (ptr, idx, val), (trow, tcol, tval), info
