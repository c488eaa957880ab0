"""Adjoint of the user half-sweep on the GPU (als_user_halfsweep_adjoint) against the FP64 host
reference gradient, through the test-only torch.autograd.Function wrapper.

The GPU runs the forward solve and the reverse pass in FP32 (atomic FP32 scatter into dL/dY), so
it is compared with the FP64 reference gradient at FP32 tolerance; the FP64 reference itself is
checked against FP64 central differences in test_oracle.py."""
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


@pytest.mark.parametrize("config,scale", [(5, 0.05), (1, 1.0)])
def test_adjoint_matches_fp64_reference(config, scale):
    torch = pytest.importorskip("torch")
    tr, te, info = ca.synth_generate(config, scale=scale)
    m, n, f, lam = info["m"], info["n"], info["f"], info["lambda"]
    csr = (tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals)
    held = (te.h_coo_row_idxs, te.h_csr_coo_col_idxs, te.h_csr_coo_vals)
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
    model.close()
