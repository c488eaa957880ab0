"""The srand(0) factor initialisation (als_model.cu:1772-1784) generated on the GPU: glibc's
rand() sequence by jump-ahead, one thread per block of 1,984 calls.  Bit-exact against the
oracle, which calls the C library's srand(0) / rand() itself, at sizes around the block edges
and at workload 4's full table (480,189 x 128 = 61.5M calls)."""
from __future__ import annotations

import numpy as np
import pytest

import cuda_als_gb300 as ca
from oracle import oracle as O

pytestmark = pytest.mark.gpu

S = 31 * 64  # rand() calls per GPU thread


@pytest.mark.parametrize("n,f", [(1, 1), (7, 5), (1, 30), (1, 31), (1, 32), (S - 1, 1), (S, 1),
                                 (S + 1, 1), (1000, 33), (3 * S + 5, 1), (480189, 128)])
def test_gpu_init_is_the_c_library_sequence(n, f):
    m = 3
    ptr = np.array([0, 1, 1, 2], np.int32)
    idx = np.array([0, n - 1], np.int32)
    val = np.array([4.0, 3.0], np.float32)
    tr = ca.host_sparse_matrix(m, n, 2).set_csr(ptr, idx, val)
    with ca.als_model(tr, None, f, 0.05, 1, precision=int(ca.PRECISION.FP32)) as mdl:
        mdl.set_factors(np.ones((m, f), np.float32), None)
        mdl.init_factors()
        U, V = mdl.get_factors()
    Ue, Ve = O.init_factors(m, n, f)
    assert not U.any()
    assert np.array_equal(V.view(np.uint32), Ve.view(np.uint32))
