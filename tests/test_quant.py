"""The FP8 table restatement (oracle/quant.py) on the CPU: e4m3 rounding against torch's
float8_e4m3fn conversion, and the scale rule."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import quant


def test_e4m3_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    if not hasattr(torch, "float8_e4m3fn"):
        pytest.skip("no float8_e4m3fn in this torch")
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.standard_normal(200000) * s for s in (1e-3, 0.05, 1.0, 30.0, 200.0)])
    x = np.clip(x, -448, 448).astype(np.float32)
    # every e4m3 value and the midpoints between neighbours (the ties)
    grid = torch.arange(256, dtype=torch.uint8).view(torch.float8_e4m3fn).float().numpy()
    grid = np.unique(grid[np.isfinite(grid)])
    mids = ((grid[1:].astype(np.float64) + grid[:-1]) / 2).astype(np.float32)
    x = np.concatenate([x, grid, mids])
    want = torch.from_numpy(x).to(torch.float8_e4m3fn).float().numpy()
    assert np.array_equal(quant.e4m3_round(x), want)


def test_scales_put_every_column_in_range():
    rng = np.random.default_rng(1)
    Y = (rng.standard_normal((1000, 37)) * np.logspace(-8, 8, 37)).astype(np.float32)
    Y[:, 5] = 0.0
    Yq, d = quant.e4m3_table(Y)
    m = np.abs(Y).max(axis=0)
    ok = m > 0
    assert np.all(m[ok] / d[ok] <= 448.0) and np.all(m[ok] / d[ok] > 224.0)
    assert d[5] == 1.0 and not Yq[:, 5].any()
    assert np.all(np.log2(d) == np.round(np.log2(d)))  # powers of two
    # three mantissa bits: relative rounding error at most 2^-4 on the normal range
    big = np.abs(Y) / d[None, :] >= 2.0 ** -6
    rel = np.abs(Yq - Y)[big] / np.abs(Y)[big]
    assert rel.max() <= 2.0 ** -4 + 1e-7
