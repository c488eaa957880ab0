"""The FP8 (e4m3) factor table the tensor-core sweep gathers, restated in numpy.  TEST
INFRASTRUCTURE.

The reference rounds its factor tables to 16 bits before its tensor-core Gram (float2half_array,
als_model.cu:54-60); the FP8 sweep rounds them to e4m3 with one power-of-two scale per feature:
d_j = 2^e_j, e_j the smallest exponent with max_r |Y_rj| / d_j <= 448 (e4m3's largest finite
value), q_rj = e4m3(Y_rj / d_j) rounded to nearest even.  Q * d (exact in FP32) is the table the
FP8 Gram sees; with it the FP64 oracle gives the FP8 sweep's answer up to FP32 accumulation.
"""
from __future__ import annotations

import numpy as np

E4M3_MAX = 448.0


def scale_exponents(Y: np.ndarray) -> np.ndarray:
    """Per-column e_j from the bit pattern of max |Y_.j| (as the quantise kernel derives it)."""
    mx = np.abs(np.asarray(Y, np.float32)).max(axis=0) if len(Y) else np.zeros(Y.shape[1],
                                                                             np.float32)
    bits = mx.astype(np.float32).view(np.uint32).astype(np.int64)
    E = ((bits >> 23) & 0xFF) - 127
    mant = bits & 0x7FFFFF
    e = np.where(mant <= 0x600000, E - 8, E - 7)
    e = np.where(bits == 0, 0, e)
    return np.clip(e, -126, 127).astype(np.int64)


def e4m3_round(x) -> np.ndarray:
    """Round to the nearest e4m3 value (ties to even), saturating at +-448; float32 out."""
    x = np.asarray(x, np.float64)
    a = np.abs(x)
    _, ex = np.frexp(a)            # a = m 2^ex, m in [0.5, 1): floor(log2 a) = ex - 1
    qe = np.maximum(ex - 1, -6) - 3  # 3 mantissa bits; subnormal quantum 2^-9
    q = np.ldexp(1.0, qe)
    r = np.minimum(np.rint(a / q) * q, E4M3_MAX)
    return np.where(a == 0, 0.0, np.sign(x) * r).astype(np.float32)


def e4m3_table(Y):
    """-> (Y' = e4m3(Y / d) * d as float32, d as float32): the values the FP8 Gram uses."""
    Y = np.asarray(Y, np.float32)
    e = scale_exponents(Y)
    d = np.ldexp(np.float64(1.0), e)
    Q = e4m3_round(Y.astype(np.float64) / d[None, :])
    return (Q.astype(np.float64) * d[None, :]).astype(np.float32), d.astype(np.float32)
