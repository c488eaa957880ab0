"""Golden outputs of the reference's own CUDA path on workload 1 (run on a GPU).

Runs the reference's half-sweep (`oracle/refkernels.py`: its `calculate_vtvs` Gram kernel and its
`updateXWithCGKernel`, built from its sources into cubins, and cuBLAS batched LU without pivoting
as `LU_solve_U` calls it) on the seeded workload 1 (1,000 x 500, 18,000 training ratings) and
writes `refkernels_workload1.npz` beside this script:

* `gram_rows`, `gram`: the reference's Gram of 16 rows at f = 10 from the srand(0) item factors;
* `lu_half_U`: one U half-sweep at f = 10 (LU) from the srand(0) init;
* `lu_U`, `lu_V`, `lu_rmse`: 10 iterations of training at f = 10 (LU), test RMSE;
* `cg_half_U`: one U half-sweep at f = 32 (CG, 6 steps, warm start from U = 0);
* `cg_V`, `cg_rmse`: 10 iterations of training at f = 32 (CG), V and test RMSE.

The CPU tests check the oracle against these (`tests/test_refpin.py`).  Usage, on a machine with
a GPU and the cubins built: python tests/golden/make_refkernel_fixtures.py [out.npz]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import cuda_als_gb300 as ca  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oracle import refkernels as RK  # noqa: E402


def main(out: Path) -> None:
    assert RK.available(), "reference cubins missing: run oracle/build.py where the reference is"
    tr, te, info = ca.synth_generate(1)
    m, n, lam = info["m"], info["n"], info["lambda"]
    csr = (tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals)
    csc = O.csr_to_csc(m, n, *csr)
    test = (te.h_coo_row_idxs, te.h_csr_coo_col_idxs, te.h_csr_coo_vals)
    res = {}
    f = 10
    U0, V0 = O.init_factors(m, n, f)
    rows = np.arange(0, m, m // 16)[:16].astype(np.int32)
    G = RK.gram(*csr[:2], V0, f, lam)
    res["gram_rows"], res["gram"] = rows, G[rows]
    res["lu_half_U"] = RK.half_sweep(*csr, V0, U0, f, lam, "lu")
    U, V = RK.train(m, n, f, lam, 10, csr, csc, "lu")
    res["lu_U"], res["lu_V"] = U, V
    res["lu_rmse"] = np.float64(O.rmse(*test, U, V))
    f = 32
    U0, V0 = O.init_factors(m, n, f)
    res["cg_half_U"] = RK.half_sweep(*csr, V0, U0, f, lam, "cg")
    U, V = RK.train(m, n, f, lam, 10, csr, csc, "cg")
    res["cg_V"] = V
    res["cg_rmse"] = np.float64(O.rmse(*test, U, V))
    np.savez_compressed(out, **res)
    print("wrote", out, {k: v.shape for k, v in res.items()})


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).with_name("refkernels_workload1.npz"))
