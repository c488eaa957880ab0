"""Shared fixtures.  Tests marked `gpu` need a CUDA device and the built libals_gb300.so; the
rest run on the CPU (oracle vs golden vectors, host logic, ABI exports, gloo ranks)."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")
    config.addinivalue_line("markers", "slow: longer-running case")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the CUDA library (nvcc cross-compiles without a GPU) and the oracle once."""
    from cuda_als_gb300 import build as b
    from oracle import build as ob

    b.build()
    ob.build()


def load_toy(name: str) -> dict:
    z = np.load(GOLDEN / f"{name}.npz")
    d = {k: z[k] for k in z.files}
    d["m"], d["n"] = int(d["m"]), int(d["n"])
    return d


@pytest.fixture(params=["toy_data", "toy_data_2"])
def toy(request):
    return load_toy(request.param)


def random_csr(rng, m, n, density=None, degrees=None, empty_rows=(), values=(1, 5)):
    """Random CSR with sorted unique columns per row (numpy only)."""
    ptr = [0]
    cols, vals = [], []
    for u in range(m):
        if u in empty_rows:
            d = 0
        elif degrees is not None:
            d = int(degrees[u])
        else:
            d = int(rng.binomial(n, density))
        d = min(d, n)
        c = np.sort(rng.choice(n, size=d, replace=False)) if d else np.zeros(0, np.int64)
        cols.append(c)
        vals.append(rng.integers(values[0], values[1] + 1, size=d).astype(np.float32))
        ptr.append(ptr[-1] + d)
    return (np.array(ptr, np.int32), np.concatenate(cols).astype(np.int32),
            np.concatenate(vals).astype(np.float32))
