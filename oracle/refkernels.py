"""The reference's own half-sweep on the GPU, for pinning.  TEST INFRASTRUCTURE ONLY.

Runs, on the current CUDA device, what `als_model::train` (als_model.cu:1766-2289) runs for its
SIMPLE Gram type:

* the right-hand side `b_u = sum_i r_ui y_i` (als_model.cu:1816-1852: cusparseScsrmm2 + geam;
  csrmm2 was removed in CUDA 11, so its successor cuSPARSE SpMM, through torch's CSR matmul);
* the Gram kernel `calculate_vtvs` (als_model.cu:91-167) itself, launched <<<rows, f>>> as
  als_model.cu:1979 does, from a device-only cubin built from the reference's source
  (`oracle/build.py` build_ref_cubins);
* then either cublasSgetrfBatched + cublasSgetrsBatched without pivoting on those Grams
  (`LU_solve_U`, als_model.cu:1570-1644), or the CG kernel `updateXWithCGKernel`
  (cumf_als_cg/cg.cu:37-232) itself, launched <<<rows, f, (4f+4) floats>>> with 6 steps as
  cg.cu:683 and als_model.cu:2006 do, warm-started from the current factors.

`train` adds the srand(0) init (als_model.cu:1772-1777) and the U-then-V order.  The CG kernel
reduces with full-warp shuffles and one atomicAdd per warp: f must be a multiple of 32 (a partial
warp is undefined), and f <= 64 keeps the two-warp atomic sums order-independent.  The kernels
index the Gram buffer with int (`blockIdx.x * f * f`), so every launch covers at most
`batch_rows(f)` rows (2^31 / f^2; the reference splits its rows into m_batches / n_batches and
passes the batch offset, als_model.cu:1891-1896): one launch of 480,189 rows at f = 100 would
write below the buffer.

Only tests/ and the timing script beside it (oracle/ref_cuda_epoch.py) import this module.  The
cubins are built where the reference tree is present and travel with the repository; without them
`available()` is False.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
from pathlib import Path

import numpy as np

from . import build as _build

CG_ITER = 6  # als_model.cu:16
SMEM_COL_CNT = 32  # main.cpp:43
# calculate_vtvs(float*, int*, int*, float, int, int, float*, int)
GRAM_KERNEL = b"_Z14calculate_vtvsPfPiS0_fiiS_i"
# calculate_vtvs_smem_row_major(float*, int*, int*, float, int, int, float*, int, int)
GRAM_SMEM_KERNEL = b"_Z29calculate_vtvs_smem_row_majorPfPiS0_fiiS_ii"
# updateXWithCGKernel(float*, float*, float*, int, int, float)
CG_KERNEL = b"_Z19updateXWithCGKernelPfS_S_iif"

_state = {}


def batch_rows(f: int) -> int:
    """Rows per launch that keep the kernels' int Gram offsets (blockIdx.x * f * f) in range."""
    return (2**31 - 1) // (f * f)


def cubins() -> dict:
    return {k: dst for k, (_, dst) in _build.REF_CUBINS.items() if dst.exists()}


def available() -> bool:
    return set(cubins()) == {"model", "cg"}


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"{what} failed with status {rc}")


def _cuda():
    if "cuda" not in _state:
        import torch

        torch.zeros(1, device="cuda")  # the runtime's primary context, current on this thread
        cu = C.CDLL("libcuda.so.1")
        mods = {}
        for key, path in cubins().items():
            image = Path(path).read_bytes()
            mod = C.c_void_p()
            _check(cu.cuModuleLoadData(C.byref(mod), C.c_char_p(image)), f"cuModuleLoadData({key})")
            mods[key] = (mod, image)
        fns = {}
        for key, mod, name in (("model", "model", GRAM_KERNEL), ("smem", "model", GRAM_SMEM_KERNEL),
                               ("cg", "cg", CG_KERNEL)):
            fn = C.c_void_p()
            _check(cu.cuModuleGetFunction(C.byref(fn), mods[mod][0], name), "cuModuleGetFunction")
            fns[key] = fn
        _state["cuda"] = (cu, mods, fns)
    return _state["cuda"]


def _cublas():
    if "cublas" not in _state:
        import torch

        names = ["libcublas.so.13", "libcublas.so"]
        for d in [os.path.dirname(torch.__file__) + "/lib", "/usr/local/cuda/lib64"] + glob.glob(
                os.path.dirname(os.path.dirname(torch.__file__)) + "/nvidia/cu*/lib"):
            names += sorted(glob.glob(d + "/libcublas.so*"))
        lib = None
        for n in names:
            try:
                lib = C.CDLL(n)
                break
            except OSError:
                continue
        if lib is None:
            raise RuntimeError("cuBLAS not found")
        h = C.c_void_p()
        _check(lib.cublasCreate_v2(C.byref(h)), "cublasCreate")
        _state["cublas"] = (lib, h)
    return _state["cublas"]


def _launch(fn, grid, block, smem, args):
    import torch

    cu = _cuda()[0]
    holders = []
    for a in args:
        if isinstance(a, torch.Tensor):
            holders.append(C.c_void_p(a.data_ptr()))
        elif isinstance(a, float):
            holders.append(C.c_float(a))
        else:
            holders.append(C.c_int(int(a)))
    params = (C.c_void_p * len(holders))(*[C.addressof(h) for h in holders])
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    u = C.c_uint
    _check(cu.cuLaunchKernel(fn, u(grid), u(1), u(1), u(block), u(1), u(1), u(smem), stream,
                             params, None), "cuLaunchKernel")


def gram(ptr, idx, Y, f, lam):
    """calculate_vtvs over every row: (rows, f, f) FP32, A_u = Y_u^T Y_u + lambda n_u I."""
    import torch

    dev = torch.device("cuda")
    d_ptr = torch.as_tensor(np.ascontiguousarray(ptr, np.int32), device=dev)
    d_idx = torch.as_tensor(np.ascontiguousarray(idx, np.int32), device=dev)
    d_Y = torch.as_tensor(np.ascontiguousarray(Y, np.float32), device=dev)
    rows = len(ptr) - 1
    assert rows <= batch_rows(f), "one launch: the kernel's int Gram offsets"
    vtvs = torch.zeros(rows * f * f, dtype=torch.float32, device=dev)
    _launch(_cuda()[2]["model"], rows, f, 0, [vtvs, d_ptr, d_idx, float(lam), rows, f, d_Y, 0])
    torch.cuda.synchronize()
    # column-major per row (vtvs[row f f + r + c f]); the Gram is symmetric
    return vtvs.view(rows, f, f).transpose(1, 2).cpu().numpy()


def m_batches_for(rows: int, f: int) -> int:
    """Fewest batches whose first (largest) batch keeps the Gram kernel's int offsets in range."""
    return max(1, -(-rows // batch_rows(f)))


def half_sweep(ptr, idx, val, Y, X, f, lam, solve="lu", m_batches=None):
    """One half-sweep as the reference runs it; returns the new X (rows x f, FP32).  Rows go in
    `m_batches` contiguous batches split as als_model.cu:1891-1896 splits them (first batches
    (rows - 1) / m_batches + 1 rows, the last the rest), each with its Gram launch at the batch
    offset and its own batched solve; by default the fewest batches the int offsets allow."""
    import torch

    dev = torch.device("cuda")
    rows, n = len(ptr) - 1, Y.shape[0]
    d_ptr = torch.as_tensor(np.ascontiguousarray(ptr, np.int32), device=dev)
    d_idx = torch.as_tensor(np.ascontiguousarray(idx, np.int32), device=dev)
    d_val = torch.as_tensor(np.ascontiguousarray(val, np.float32), device=dev)
    d_Y = torch.as_tensor(np.ascontiguousarray(Y, np.float32), device=dev)
    R = torch.sparse_csr_tensor(d_ptr, d_idx, d_val, size=(rows, n))
    B = (R @ d_Y).contiguous()  # rows x f: b_u contiguous per row (the reference's VTRT)
    nb = m_batches or m_batches_for(rows, f)
    first = (rows - 1) // nb + 1
    assert first <= batch_rows(f), "one launch: the kernel's int Gram offsets"
    vtvs = torch.zeros(first * f * f, dtype=torch.float32, device=dev)
    if solve == "cg":
        assert f % 32 == 0 and f <= 64, "the reference CG kernel needs whole warps (f = 32, 64)"
        d_X = torch.as_tensor(np.ascontiguousarray(X, np.float32), device=dev).clone()
    elif solve != "lu":
        raise ValueError(solve)
    for k in range(nb):
        off = k * first
        bs = min(first, rows - off)
        if bs <= 0:
            break
        vtvs.zero_()
        _launch(_cuda()[2]["model"], bs, f, 0, [vtvs, d_ptr, d_idx, float(lam), rows, f, d_Y, off])
        if solve == "lu":
            lib, h = _cublas()
            stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
            _check(lib.cublasSetStream_v2(h, stream), "cublasSetStream")
            a_ptrs = torch.arange(bs, dtype=torch.int64, device=dev) * (f * f * 4) + vtvs.data_ptr()
            b_ptrs = (torch.arange(bs, dtype=torch.int64, device=dev) * (f * 4) + B.data_ptr() +
                      off * f * 4)
            infos = torch.zeros(bs, dtype=torch.int32, device=dev)
            vp = C.c_void_p
            _check(lib.cublasSgetrfBatched(h, C.c_int(f), vp(a_ptrs.data_ptr()), C.c_int(f), None,
                                           vp(infos.data_ptr()), C.c_int(bs)), "cublasSgetrfBatched")
            info = C.c_int(0)
            _check(lib.cublasSgetrsBatched(h, C.c_int(0), C.c_int(f), C.c_int(1),
                                           vp(a_ptrs.data_ptr()), C.c_int(f), None,
                                           vp(b_ptrs.data_ptr()), C.c_int(f), C.byref(info),
                                           C.c_int(bs)), "cublasSgetrsBatched")
        else:
            _launch(_cuda()[2]["cg"], bs, f, (4 * f + 4) * 4,
                    [vtvs, d_X[off:off + bs], B[off:off + bs], bs, f, float(CG_ITER)])
    torch.cuda.synchronize()
    return (B if solve == "lu" else d_X).cpu().numpy()


def train(m, n, f, lam, iters, csr, csc, solve="lu", m_batches=None, n_batches=None):
    """srand(0) init, then iters x (U over the CSR, V over the CSC) -> (U, V)."""
    from . import oracle as O

    U, V = O.init_factors(m, n, f)
    for _ in range(iters):
        U = half_sweep(csr[0], csr[1], csr[2], V, U, f, lam, solve, m_batches)
        V = half_sweep(csc[0], csc[1], csc[2], U, V, f, lam, solve, n_batches)
    return U, V


class Epoch:
    """The reference's LU path for one workload, resident on the GPU, for timing: per half-sweep
    the right-hand side (cuSPARSE SpMM), the zeroed Gram buffer and `calculate_vtvs_smem_row_major`
    (als_model.cu:169-241, the shared-memory FP32 Gram, launched <<<rows, f, smem_col_cnt f
    floats>>> as als_model.cu:1900 does, with main.cpp's smem_col_cnt = 32), then cuBLAS batched
    LU without pivoting; rows in batches of at most `batch_rows(f)` (the kernel's int offsets),
    each with its batch offset, as the reference's m_batches / n_batches loop does."""

    def __init__(self, m, n, f, lam, csr, csc):
        import torch

        dev = torch.device("cuda")
        self.f, self.lam = f, float(lam)
        self.sides = []
        for (ptr, idx, val), rows, cols in ((csr, m, n), (csc, n, m)):
            d_ptr = torch.as_tensor(np.ascontiguousarray(ptr, np.int32), device=dev)
            d_idx = torch.as_tensor(np.ascontiguousarray(idx, np.int32), device=dev)
            d_val = torch.as_tensor(np.ascontiguousarray(val, np.float32), device=dev)
            R = torch.sparse_csr_tensor(d_ptr, d_idx, d_val, size=(rows, cols))
            self.sides.append((rows, d_ptr, d_idx, R))
        self.batch = min(max(m, n), batch_rows(f))
        self.vtvs = torch.zeros(self.batch * f * f, dtype=torch.float32, device=dev)
        self.a_ptrs = (torch.arange(self.batch, dtype=torch.int64, device=dev) * (f * f * 4) +
                       self.vtvs.data_ptr())
        self.infos = torch.zeros(self.batch, dtype=torch.int32, device=dev)
        U0, V0 = _init(m, n, f)
        self.X = [torch.as_tensor(U0, device=dev), torch.as_tensor(V0, device=dev)]

    def half(self, side):
        import torch

        f = self.f
        rows, d_ptr, d_idx, R = self.sides[side]
        Y = self.X[1 - side]
        B = (R @ Y).contiguous()
        lib, h = _cublas()
        _check(lib.cublasSetStream_v2(h, C.c_void_p(torch.cuda.current_stream().cuda_stream)),
               "cublasSetStream")
        vp = C.c_void_p
        for off in range(0, rows, self.batch):
            bs = min(self.batch, rows - off)
            self.vtvs[: bs * f * f].zero_()
            _launch(_cuda()[2]["smem"], bs, f, SMEM_COL_CNT * f * 4,
                    [self.vtvs, d_ptr, d_idx, self.lam, rows, f, Y, SMEM_COL_CNT, off])
            b_ptrs = (torch.arange(bs, dtype=torch.int64, device=B.device) * (f * 4) +
                      B.data_ptr() + off * f * 4)
            _check(lib.cublasSgetrfBatched(h, C.c_int(f), vp(self.a_ptrs.data_ptr()), C.c_int(f),
                                           None, vp(self.infos.data_ptr()), C.c_int(bs)),
                   "getrfBatched")
            info = C.c_int(0)
            _check(lib.cublasSgetrsBatched(h, C.c_int(0), C.c_int(f), C.c_int(1),
                                           vp(self.a_ptrs.data_ptr()), C.c_int(f), None,
                                           vp(b_ptrs.data_ptr()), C.c_int(f), C.byref(info),
                                           C.c_int(bs)), "getrsBatched")
        self.X[side] = B

    def epoch(self):
        self.half(0)
        self.half(1)


def _init(m, n, f):
    from . import oracle as O

    return O.init_factors(m, n, f)
