"""nnz buckets, the Cholesky/CG autotuner (ALS_SOLVE_AUTO) and CUDA-graph epochs, through the C ABI.

Workload 2's shape (lognormal row degrees, Zipf columns, f = 64): the buckets must
equal the host's degree counts exactly, the tuner's choice must follow its rule from its own
measurements, training under AUTO must reach the plain-FP32 Cholesky test RMSE, and an epoch
replayed from the captured graph must give the same bits as the same epoch launched eagerly.
"""
from __future__ import annotations

import numpy as np
import pytest

import cuda_als_gb300 as ca

pytestmark = pytest.mark.gpu

AUTO_TOL = 5e-2             # the tuner's CG-vs-Cholesky agreement bound (sweep.cpp)
CG16_MARGIN = 0.85          # the lead it asks of the tensor-core CG (sweep.cpp)
TOL_RMSE = 2e-3          # test RMSE after training vs plain FP32 Cholesky


def workload2(scale=0.1):
    tr, te, info = ca.synth_generate(2, scale=scale)
    return tr, te, info


def model(tr, te, info, solve, precision, iters=10, **opt):
    return ca.als_model(tr, te, info["f"], info["lambda"], iters,
                        ca.CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR, solve, precision=int(precision),
                        **opt)


def expected_cuts(ptr, f):
    deg = np.diff(np.asarray(ptr, np.int64))
    heavy = int((deg >= 8 * f).sum())
    mid = int(((deg >= f) & (deg < 8 * f)).sum())
    cuts = [0, heavy, heavy + mid]
    los = [c for k, c in enumerate(cuts) if (cuts + [len(deg)])[k + 1] > c]
    return los


@pytest.mark.parametrize("precision", [ca.PRECISION.BF16, ca.PRECISION.FP32])
def test_auto_buckets_follow_degrees_and_tuner_rule(precision):
    tr, te, info = workload2()
    f = info["f"]
    ptr_u = tr.h_csr_row_ptrs
    cptr = np.zeros(info["n"] + 1, np.int64)
    np.add.at(cptr, tr.h_csr_coo_col_idxs.astype(np.int64) + 1, 1)
    ptr_v = np.cumsum(cptr)
    with model(tr, te, info, ca.SOLVE_TYPE.AUTO, precision, iters=3) as mdl:
        mdl.init_factors()
        mdl.iterate(3)
        for side, ptr in ((0, ptr_u), (1, ptr_v)):
            plan = mdl.plan(side)
            assert [b["lo"] for b in plan] == expected_cuts(ptr, f)
            tuning = mdl.tuning(side)
            assert len(tuning) == len(plan)
            for b, t in zip(plan, tuning):
                assert t["ms_cg"] > 0 and t["ms_cholesky"] > 0 and t["rel_diff"] >= 0
                # the FP16-Gram CG (products on the tensor core) is a candidate on that path only
                tc = precision != ca.PRECISION.FP32
                assert (t["ms_cg16"] > 0 and t["rel_diff_cg16"] >= 0) if tc else t["ms_cg16"] < 0
                cands = [(t["ms_cholesky"], ca.SOLVE_TYPE.CHOLESKY)]
                if t["rel_diff"] <= AUTO_TOL:
                    cands.append((t["ms_cg"], ca.SOLVE_TYPE.CUMF_ALS_CG_FP32))
                best = min(cands, key=lambda c: c[0])
                # the tensor-core CG needs a 15% lead (its larger fixed cost per row)
                if tc and t["rel_diff_cg16"] <= AUTO_TOL and t["ms_cg16"] < CG16_MARGIN * best[0]:
                    best = (t["ms_cg16"], ca.SOLVE_TYPE.CUMF_ALS_CG_FP16)
                assert b["solver"] == best[1]
                assert b["kind"] == (0 if precision == ca.PRECISION.FP32 else 1)
        assert mdl.counters()["flagged_rows"] == 0


def test_fixed_solver_is_one_bucket():
    tr, te, info = workload2()
    with model(tr, te, info, ca.SOLVE_TYPE.CHOLESKY, ca.PRECISION.BF16, iters=1) as mdl:
        mdl.init_factors()
        mdl.iterate(2)
        for side in (0, 1):
            assert mdl.plan(side) == [{"lo": 0, "kind": 1, "solver": int(ca.SOLVE_TYPE.CHOLESKY)}]
            assert all(t["ms_cg"] < 0 for t in mdl.tuning(side))


@pytest.mark.parametrize("config,scale", [(2, 0.1), (3, 0.05)])
def test_auto_plan_launches_one_kernel_per_solver_run(config, scale):
    """Adjacent buckets that settled on the same solver are contiguous rows of the order and share
    one launch: an epoch's kernel count is one BF16 quantise per side plus one launch per run of
    equal solvers in each side's plan (f = 64 and f = 100)."""
    tr, te, info = ca.synth_generate(config, scale=scale)
    with model(tr, te, info, ca.SOLVE_TYPE.AUTO, ca.PRECISION.BF16, iters=3) as mdl:
        mdl.init_factors()
        mdl.iterate(3)  # the tuning sweeps are over: the plan is final
        mdl.iterate(1)
        expected = 0
        for side in (0, 1):
            solvers = [b["solver"] for b in mdl.plan(side)]
            expected += 1 + sum(1 for k in range(len(solvers))
                                if k == 0 or solvers[k] != solvers[k - 1])
        assert mdl.counters()["launches"] == expected


@pytest.mark.parametrize("config,precision", [(2, ca.PRECISION.BF16), (2, ca.PRECISION.FP32),
                                              (5, ca.PRECISION.BF16)])
def test_auto_training_reaches_fp32_cholesky_rmse(config, precision):
    """Full-size workload 2 (69,878 x 10,677, 10M ratings, f = 64) and 5 (283,228 x 58,098, 24.3M
    ratings, f = 128, whose items lighter than f take CG under the tuner's agreement bound), 10
    iterations.  (Scaled-down copies over-fit, test RMSE ~1.34, where 6-step CG itself lands 2e-3
    from Cholesky.)"""
    tr, te, info = ca.synth_generate(config, scale=1.0)
    with model(tr, te, info, ca.SOLVE_TYPE.CHOLESKY, ca.PRECISION.FP32) as ref:
        ref.train()
        r_ref = ref.rsme_test()
    with model(tr, te, info, ca.SOLVE_TYPE.AUTO, precision) as mdl:
        mdl.train()
        r = mdl.rsme_test()
    assert abs(r - r_ref) < TOL_RMSE


@pytest.mark.parametrize("precision,solve", [
    (ca.PRECISION.BF16, ca.SOLVE_TYPE.CHOLESKY),
    (ca.PRECISION.BF16, ca.SOLVE_TYPE.AUTO),
    (ca.PRECISION.FP32, ca.SOLVE_TYPE.CUMF_ALS_CG_FP32),
])
def test_graph_epochs_match_eager_bits(precision, solve):
    """Rows are independent and each row's arithmetic has a fixed order, so an epoch replayed from
    the captured graph must reproduce the same epoch launched eagerly (half_sweep U, then V) bit
    for bit, from the same factors and with the same plan (one handle: under AUTO the plan comes
    from timings, so two handles may tune differently)."""
    tr, te, info = workload2()
    with model(tr, te, info, solve, precision, use_graph=1) as mdl:
        mdl.init_factors()
        mdl.iterate(4)                      # plan final (tuned under AUTO), epoch captured
        U0, V0 = mdl.get_factors()
        mdl.iterate(1)                      # replayed
        Ug, Vg = mdl.get_factors()
        mdl.set_factors(U0, V0)
        mdl.half_sweep(0)                   # eager
        mdl.half_sweep(1)
        Ue, Ve = mdl.get_factors()
    assert np.array_equal(Ug, Ue) and np.array_equal(Vg, Ve)
    if solve != ca.SOLVE_TYPE.AUTO:         # a fixed plan: a handle without graphs agrees too
        with model(tr, te, info, solve, precision, use_graph=0) as mdl:
            mdl.set_factors(U0, V0)
            mdl.iterate(1)
            Un, Vn = mdl.get_factors()
        assert np.array_equal(Ug, Un) and np.array_equal(Vg, Vn)


def test_graph_survives_value_update_and_reload():
    """update_values keeps the captured epoch (same buffers); reload drops it and rebuilds the
    buckets; both must match a fresh model on the new data."""
    tr, te, info = workload2()
    vals2 = (tr.h_csr_coo_vals[::-1]).copy()
    with model(tr, te, info, ca.SOLVE_TYPE.CHOLESKY, ca.PRECISION.BF16) as mdl:
        mdl.init_factors()
        mdl.iterate(3)
        mdl.update_values(vals2)
        mdl.init_factors()
        mdl.iterate(3)
        got = mdl.get_factors()
    tr2 = ca.host_sparse_matrix(info["m"], info["n"], len(vals2)).set_csr(
        tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, vals2)
    with model(tr2, te, info, ca.SOLVE_TYPE.CHOLESKY, ca.PRECISION.BF16) as mdl:
        mdl.init_factors()
        mdl.iterate(3)
        want = mdl.get_factors()
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
