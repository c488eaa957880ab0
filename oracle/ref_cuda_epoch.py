"""Time the reference's own CUDA path (its shared-memory FP32 Gram kernel + cuBLAS batched LU,
`refkernels.Epoch`) on a synthetic workload, on the current GPU.  TEST INFRASTRUCTURE.

    python -m oracle.ref_cuda_epoch [--config 3] [--scale 1.0] [--iters 10]

Prints one JSON line: ms per epoch (CUDA events over `iters` epochs after one warm-up epoch,
inputs resident) and the test RMSE after the warm-up + `iters` epochs.
"""
from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))


def main() -> None:
    import torch

    import cuda_als_gb300 as ca
    from oracle import oracle as O
    from oracle import refkernels as RK

    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, default=3)
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--iters", type=int, default=10)
    a = ap.parse_args()
    tr, te, info = ca.synth_generate(a.config, scale=a.scale)
    m, n, f, lam = info["m"], info["n"], info["f"], info["lambda"]
    csr = (tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals)
    csc = O.csr_to_csc(m, n, *csr)
    ep = RK.Epoch(m, n, f, lam, csr, csc)
    ep.epoch()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.iters - 1):
        ep.epoch()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / max(a.iters - 1, 1)
    U, V = ep.X[0].cpu().numpy(), ep.X[1].cpu().numpy()
    test = (te.h_coo_row_idxs, te.h_csr_coo_col_idxs, te.h_csr_coo_vals)
    print(json.dumps({"workload": a.config, "scale": a.scale, "m": m, "n": n, "f": f,
                      "path": "reference CUDA: calculate_vtvs_smem_row_major + cuBLAS "
                              "getrf/getrsBatched (LU), cuSPARSE SpMM right-hand side",
                      "ms_per_epoch": round(ms, 3),
                      "test_rmse_after_iters": O.rmse(*test, U, V), "iters": a.iters}))


if __name__ == "__main__":
    main()
