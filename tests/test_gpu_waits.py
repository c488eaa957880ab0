"""The tensor-core sweep's bounded device waits, made to run out on purpose.

Every spin-wait of the sweep kernel (a stage's gathered rows, a free accumulator, a finished Gram,
a product on the tensor core, a free metadata slot) is bounded by the handle's wait limit; the
drains at the end of a CTA keep their own 10 s bound.  With the limit set to 1 ns, the first wait
that is not met within 16 tries runs out: its CTA raises the abort flag, every role stops taking
work, lets the copies and MMAs it issued land, frees its tensor memory and returns, and the call
fails with ALS_ERR_TIMEOUT.  No fault and no hang is involved: the waits are healthy ones, given
no time.  The same handle, back at the default limit, then reproduces a clean run bit for bit.
"""
from __future__ import annotations

import numpy as np
import pytest

import cuda_als_gb300 as ca

pytestmark = pytest.mark.gpu

CASES = [(3, 0.05, ca.SOLVE_TYPE.CHOLESKY), (3, 0.05, ca.SOLVE_TYPE.CUMF_ALS_CG_FP32),
         (3, 0.05, ca.SOLVE_TYPE.CUMF_ALS_CG_FP16), (3, 0.05, ca.SOLVE_TYPE.LU),
         (5, 0.1, ca.SOLVE_TYPE.CHOLESKY), (5, 0.1, ca.SOLVE_TYPE.CUMF_ALS_CG_FP16),
         (2, 0.1, ca.SOLVE_TYPE.CUMF_ALS_CG_FP32)]


@pytest.mark.parametrize("config,scale,solve", CASES)
def test_a_wait_that_runs_out_fails_the_call_and_the_handle_recovers(config, scale, solve):
    tr, te, info = ca.synth_generate(config, scale=scale)
    m, n, f, lam = info["m"], info["n"], info["f"], info["lambda"]
    rng = np.random.default_rng(config)
    U0 = (rng.standard_normal((m, f)) * 0.1).astype(np.float32)
    V0 = (rng.standard_normal((n, f)) * 0.3).astype(np.float32)
    with ca.als_model(tr, te, f, lam, 1, ca.CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR_TENSOR, solve,
                      precision=int(ca.PRECISION.BF16)) as mdl:
        mdl.set_factors(U0, V0)
        mdl.half_sweep(0)
        mdl.half_sweep(1)
        Uc, Vc = mdl.get_factors()
        for side in (0, 1):
            mdl.set_wait_limit_ns(1)
            mdl.set_factors(U0, V0)
            with pytest.raises(ca.ALSError) as e:
                mdl.half_sweep(side)
            assert e.value.status == ca.Status.TIMEOUT, e.value
            assert "bounded device wait ran out" in str(e.value)
        mdl.set_wait_limit_ns(0)
        mdl.set_factors(U0, V0)
        mdl.half_sweep(0)
        mdl.half_sweep(1)
        U, V = mdl.get_factors()
        assert mdl.counters()["flagged_rows"] == 0
    assert np.array_equal(U, Uc) and np.array_equal(V, Vc)


def test_an_epoch_after_a_timeout_runs_from_the_graph_again():
    """iterate() (graph-replayed epochs) after a timed-out call: the limit change drops the
    captured graph, and the epochs at the default limit equal a fresh handle's."""
    tr, te, info = ca.synth_generate(3, scale=0.05)
    f, lam = info["f"], info["lambda"]
    kw = dict(precision=int(ca.PRECISION.BF16))
    with ca.als_model(tr, te, f, lam, 3, ca.CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR_TENSOR,
                      ca.SOLVE_TYPE.CHOLESKY, **kw) as fresh:
        fresh.init_factors()
        fresh.iterate(3)
        Uf, Vf = fresh.get_factors()
    with ca.als_model(tr, te, f, lam, 3, ca.CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR_TENSOR,
                      ca.SOLVE_TYPE.CHOLESKY, **kw) as mdl:
        mdl.init_factors()
        mdl.iterate(2)  # eager epoch, then the captured graph
        mdl.set_wait_limit_ns(1)
        with pytest.raises(ca.ALSError) as e:
            mdl.iterate(1)
        assert e.value.status == ca.Status.TIMEOUT
        mdl.set_wait_limit_ns(0)
        mdl.init_factors()
        mdl.iterate(3)
        U, V = mdl.get_factors()
    assert np.array_equal(U, Uf) and np.array_equal(V, Vf)
