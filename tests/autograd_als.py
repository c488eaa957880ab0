"""Test-only torch.autograd.Function around the adjoint entry point of the C ABI.

forward(V, lam) runs the user half-sweep with item factors V (als_user_halfsweep_adjoint) and
returns the held-out squared error; backward hands back dL/dV and dL/dlambda from the same call.
Only the tests use it; the library itself has no torch dependency.
"""
from __future__ import annotations

import numpy as np


def make_function(torch, model, held):
    rows, cols, vals = held

    class ALSUserHalfSweep(torch.autograd.Function):
        @staticmethod
        def forward(ctx, V, lam):
            if float(lam) != model.lambda_:
                raise ValueError("lambda is fixed by the model configuration")
            model.set_factors(None, V.detach().cpu().numpy().astype(np.float32))
            loss, dV, dlam = model.user_halfsweep_adjoint(rows, cols, vals)
            ctx.save_for_backward(torch.from_numpy(dV).to(V.device),
                                  torch.tensor(dlam, dtype=torch.float64))
            return torch.tensor(loss, dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad):
            dV, dlam = ctx.saved_tensors
            return grad.to(dV.dtype) * dV, grad * dlam

    return ALSUserHalfSweep
