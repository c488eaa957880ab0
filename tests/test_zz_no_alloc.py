"""The allocation-free transpose entry point (als_csr_to_csc_device_noalloc).

It is for callers that may not allocate device memory: a plug-in hosted by an engine that owns
all device memory, or a latency-critical loop that must not wait on an allocator.  It keeps its scratch in one fixed array inside the library instead.  Its
output must be identical to the allocating entry point's (als_csr_to_csc_device) on every call:
this is integer and permutation work, so the comparison is bit-exact.  The file is named so that
pytest collects it last.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import cuda_als_gb300 as ca
from conftest import random_csr
from cuda_als_gb300._lib import CsrView, lib

pytestmark = pytest.mark.gpu


def _transpose(fn, torch, m, n, ptr, idx, val):
    dev = torch.device("cuda", 0)
    d_ptr = torch.from_numpy(np.ascontiguousarray(ptr, np.int32)).to(dev)
    d_idx = torch.from_numpy(np.ascontiguousarray(idx, np.int32)).to(dev)
    d_val = torch.from_numpy(np.ascontiguousarray(val, np.float32)).to(dev)
    o_ptr = torch.full((n + 1,), -7, dtype=torch.int32, device=dev)
    o_idx = torch.full((max(1, len(idx)),), -7, dtype=torch.int32, device=dev)
    o_val = torch.full((max(1, len(idx)),), -7.0, dtype=torch.float32, device=dev)
    view = CsrView(m, n, len(idx), d_ptr.data_ptr(), d_idx.data_ptr(), d_val.data_ptr())
    stream = torch.cuda.current_stream(dev)
    status = fn(C.byref(view), C.c_void_p(o_ptr.data_ptr()), C.c_void_p(o_idx.data_ptr()),
                C.c_void_p(o_val.data_ptr()), C.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize(dev)
    return status, o_ptr.cpu().numpy(), o_idx.cpu().numpy()[:len(idx)], o_val.cpu().numpy()[:len(idx)]


def test_noalloc_transpose_equals_allocating_transpose_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2024)
    cases = [
        (300, 5000, random_csr(rng, 300, 5000, density=0.05, empty_rows={0, 17})),
        (2000, 70000, random_csr(rng, 2000, 70000, density=0.004)),  # ~560k ratings, 3 passes
    ]
    for m, n, (ptr, idx, val) in cases:
        ref = _transpose(lib().als_csr_to_csc_device, torch, m, n, ptr, idx, val)
        assert ref[0] == 0
        for _ in range(2):  # two calls in a row share the same scratch array
            got = _transpose(lib().als_csr_to_csc_device_noalloc, torch, m, n, ptr, idx, val)
            assert got[0] == 0, lib().als_last_error(None)
            assert np.array_equal(got[1], ref[1])
            assert np.array_equal(got[2], ref[2])
            assert np.array_equal(got[3], ref[3])


def test_noalloc_transpose_rejects_inputs_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.int32, device=dev)
    view = CsrView(10, 10, 2_000_000, buf.data_ptr(), buf.data_ptr(), buf.data_ptr())
    status = lib().als_csr_to_csc_device_noalloc(C.byref(view), C.c_void_p(buf.data_ptr()),
                                                 C.c_void_p(buf.data_ptr()),
                                                 C.c_void_p(buf.data_ptr()), None)
    assert status == ca.Status.INVALID_ARG
    assert b"scratch" in lib().als_last_error(None)
