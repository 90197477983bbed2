"""BSR SpMV and deterministic dot products on the GPU (thin wrappers over the C ABI)."""
from __future__ import annotations

import numpy as np
import torch

from ._lib import check, lib, ptr


def _stream() -> int:
    return int(torch.cuda.current_stream().cuda_stream)


def _i32(a) -> torch.Tensor:
    return torch.as_tensor(np.asarray(a, dtype=np.int32) if not isinstance(a, torch.Tensor) else a,
                           dtype=torch.int32).to("cuda").contiguous()


def bsr_spmv(indptr, indices, values, block_size: int, x, *, transpose: bool = False,
             out: torch.Tensor | None = None) -> torch.Tensor:
    """``y = A x`` (or ``A^T x``) for a BSR matrix with row-major ``b x b`` blocks.

    The operator of ``_CsrOperator.apply`` (``aquaflux/solve/multigrid.py:1302-1390``); fp64 or
    fp32 chosen by the dtype of ``values`` (``x`` must match).
    """
    v = torch.as_tensor(values).to("cuda").contiguous()
    dtype = v.dtype
    if dtype not in (torch.float64, torch.float32):
        raise ValueError("values must be float64 or float32")
    xv = torch.as_tensor(x).to("cuda", dtype=dtype).contiguous()
    ip, ix = _i32(indptr), _i32(indices)
    nbr = ip.numel() - 1
    y = torch.empty(nbr * block_size, dtype=dtype, device="cuda") if out is None else out
    fn = lib().fv_bsr_spmv_f64 if dtype == torch.float64 else lib().fv_bsr_spmv_f32
    check(fn(nbr, block_size, ptr(ip), ptr(ix), ptr(v), ptr(xv), ptr(y), int(transpose), _stream()))
    return y


def dot(x: torch.Tensor, y: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """Run-to-run bit-identical fp64 dot product (fixed blocking and summation order)."""
    r = torch.empty((), dtype=torch.float64, device="cuda") if out is None else out
    check(lib().fv_dot_f64(x.numel(), ptr(x), ptr(y), ptr(r), _stream()))
    return r
