"""Adjoint of the user half-sweep on the GPU (als_user_halfsweep_adjoint and its FP64 form)
against the FP64 host reference gradient and against FP64 central differences of the GPU's own
loss, through the C ABI and the test-only torch.autograd.Function wrapper.

The FP32 entry point runs the forward solve and the reverse pass in FP32, so it is compared with
the FP64 reference gradient at FP32 tolerance; dL/dY is summed per item in a fixed order, so two
calls agree bit for bit.  The FP64 entry point runs everything in FP64: it matches the host
reference to rounding and passes central differences at 1e-5 relative."""
from __future__ import annotations

import numpy as np
import pytest

import cuda_als_gb300 as ca
from autograd_als import make_function
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL_GRAD = 2e-3   # relative Frobenius error of dL/dY, FP32 GPU vs FP64 host
TOL_LOSS = 1e-4   # relative error of the held-out loss
TOL_DLAM = 5e-3   # relative error of dL/dlambda


def _workload(config, scale):
    tr, te, info = ca.synth_generate(config, scale=scale)
    m, n, f, lam = info["m"], info["n"], info["f"], info["lambda"]
    csr = (tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals)
    held = (te.h_coo_row_idxs, te.h_csr_coo_col_idxs, te.h_csr_coo_vals)
    return tr, m, n, f, lam, csr, held


@pytest.mark.parametrize("config,scale", [(5, 0.05), (1, 1.0)])
def test_adjoint_matches_fp64_reference(config, scale):
    torch = pytest.importorskip("torch")
    tr, m, n, f, lam, csr, held = _workload(config, scale)
    rng = np.random.default_rng(config)
    V = (rng.standard_normal((n, f)) * 0.2).astype(np.float32)
    model = ca.als_model(tr, None, f, lam, 1, ca.CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR,
                         ca.SOLVE_TYPE.CHOLESKY)
    Fn = make_function(torch, model, held)
    Vt = torch.tensor(V, requires_grad=True)
    lt = torch.tensor(float(np.float32(lam)), dtype=torch.float64, requires_grad=True)
    loss = Fn.apply(Vt, lt)
    loss.backward()
    e_loss, X, G, e_dlam = O.user_adjoint(m, n, f, float(np.float32(lam)), csr, V, held)
    assert float(loss.detach()) == pytest.approx(e_loss, rel=TOL_LOSS)
    g = Vt.grad.numpy().astype(np.float64)
    assert np.linalg.norm(g - G) / np.linalg.norm(G) < TOL_GRAD
    assert float(lt.grad) == pytest.approx(e_dlam, rel=TOL_DLAM)
    # the forward solution the adjoint wrote is the user half-sweep's
    U, _ = model.get_factors()
    assert np.linalg.norm(U - X) / np.linalg.norm(X) < 1e-4
    # deterministic: a second call gives the same bits
    model.set_factors(None, V)
    l2, g2, d2 = model.user_halfsweep_adjoint(*held)
    l1, g1, d1 = model.user_halfsweep_adjoint(*held)
    assert l1 == l2 and d1 == d2 and np.array_equal(g1.view(np.uint32), g2.view(np.uint32))
    model.close()


@pytest.mark.parametrize("config,scale", [(5, 0.05), (1, 1.0)])
def test_fp64_adjoint_matches_the_host_reference_to_rounding(config, scale):
    tr, m, n, f, lam, csr, held = _workload(config, scale)
    rng = np.random.default_rng(config + 100)
    Y = rng.standard_normal((n, f)) * 0.2
    with ca.als_model(tr, None, f, lam, 1, ca.CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR,
                      ca.SOLVE_TYPE.CHOLESKY) as model:
        loss, G, dlam = model.user_halfsweep_adjoint_f64(*held, Y, lam)
        U, _ = model.get_factors()
    e_loss, X, Ge, e_dlam = O.user_adjoint(m, n, f, lam, csr, Y, held)
    assert loss == pytest.approx(e_loss, rel=1e-11)
    assert np.linalg.norm(G - Ge) / np.linalg.norm(Ge) < 1e-10
    assert dlam == pytest.approx(e_dlam, rel=1e-10)
    assert np.linalg.norm(U - X) / np.linalg.norm(X) < 1e-6  # (U holds x rounded to FP32)


def test_fp64_adjoint_passes_central_differences_on_workload5():
    """64 random coordinates of dL/dY and dL/dlambda of the held-out loss on scaled workload 5
    (MovieLens-latest shape, f = 128, 14,161 x 2,905, 61k ratings, 6k held out): the GPU's FP64
    gradient against central differences of the GPU's own FP64 loss, 1e-5 relative."""
    tr, m, n, f, lam, csr, held = _workload(5, 0.05)
    rng = np.random.default_rng(55)
    Y = rng.standard_normal((n, f)) * 0.2
    with ca.als_model(tr, None, f, lam, 1, ca.CALCULATE_VTVS_TYPE.SMEM_ROW_MAJOR,
                      ca.SOLVE_TYPE.CHOLESKY) as model:
        L = lambda Yv, lv: model.user_halfsweep_adjoint_f64(*held, Yv, lv)[0]  # noqa: E731
        loss, G, dlam = model.user_halfsweep_adjoint_f64(*held, Y, lam)
        h = 1e-4
        touched = np.unique(np.concatenate([csr[1], held[1]]))
        items = rng.choice(touched, 64, replace=False)
        ks = rng.integers(0, f, 64)
        for i, k in zip(items, ks):
            Yp, Ym = Y.copy(), Y.copy()
            Yp[i, k] += h
            Ym[i, k] -= h
            fd = (L(Yp, lam) - L(Ym, lam)) / (2 * h)
            assert G[i, k] == pytest.approx(fd, rel=1e-5, abs=1e-8), (int(i), int(k))
        hl = 1e-6
        fd = (L(Y, lam + hl) - L(Y, lam - hl)) / (2 * hl)
        assert dlam == pytest.approx(fd, rel=1e-5)
