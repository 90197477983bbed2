"""Zero-fill ILU(0) on the GPU with the reference's ``Ilu0`` interface.

Mirrors ``aquaflux/solve/ilu0.py:153-255``: construct from a square sparse operator (indices
sorted, int32), ``refactor(values)`` re-factorizes new values on the same pattern (``ValueError`` on
a length mismatch), ``solve(rhs, transpose=False)`` returns ``(LU)^-1 rhs`` (or ``(LU)^-T rhs``)
without touching ``rhs``.  A missing diagonal raises ``ValueError`` and an exactly-zero pivot
``ZeroDivisionError``, with the reference's messages (``aquaflux/solve/_ilu0.pyx:56-63, 107-111``).

Beyond the reference: ``block_size`` b > 1 factors a BSR operator with dense ``b x b`` blocks
(the cell-major interleaved Jacobian) -- the same elimination as scalar ILU(0) over the expanded
pattern -- and ``precision=32`` keeps the factor and the sweeps in fp32 (the preconditioner of
the mixed-precision Newton-Krylov solve).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from ._lib import FV_ERR_NO_DIAG, FV_ERR_ZERO_PIVOT, FvError, check, lib, ptr


def _stream() -> int:
    return int(torch.cuda.current_stream().cuda_stream)


def _raise(e: FvError):
    if e.code == FV_ERR_NO_DIAG:
        raise ValueError(e.message) from None
    if e.code == FV_ERR_ZERO_PIVOT:
        raise ZeroDivisionError(e.message) from None
    raise e


class Ilu0:
    """GPU ILU(0) factor of a fixed (block) sparsity pattern."""

    def __init__(self, matrix, *, block_size: int = 1, precision: int = 64):
        import scipy.sparse as sp

        if block_size == 1:
            csr = sp.csr_matrix(matrix)
            csr.sort_indices()
            if csr.shape[0] != csr.shape[1]:
                raise ValueError(f"ILU(0) needs a square operator, got {csr.shape}.")
            self._setup(csr.indptr, csr.indices, 1, precision)
            self.refactor(csr.data)
        else:
            bsr = sp.bsr_matrix(matrix, blocksize=(block_size, block_size))
            bsr.sort_indices()
            if bsr.shape[0] != bsr.shape[1]:
                raise ValueError(f"ILU(0) needs a square operator, got {bsr.shape}.")
            self._setup(bsr.indptr, bsr.indices, block_size, precision)
            self.refactor(bsr.data.reshape(-1))

    @classmethod
    def from_csr(cls, indptr, indices, values, *, block_size: int = 1, precision: int = 64):
        """Factor a (B)CSR operator given as arrays (``values`` of length nnzb * b * b)."""
        obj = cls.__new__(cls)
        obj._setup(indptr, indices, block_size, precision)
        obj.refactor(values)
        return obj

    def _setup(self, indptr, indices, b, precision):
        self._indptr = np.ascontiguousarray(indptr, dtype=np.int32)
        self._indices = np.ascontiguousarray(indices, dtype=np.int32)
        self._n = len(self._indptr) - 1
        self._b = int(b)
        self._precision = int(precision)
        self._dtype = torch.float64 if precision == 64 else torch.float32
        self._nvals = int(self._indptr[-1]) * b * b
        h = ctypes.c_void_p()
        try:
            check(lib().fv_ilu0_create(self._n, b, ptr(self._indptr), ptr(self._indices),
                                       self._precision, _stream(), ctypes.byref(h)))
        except FvError as e:
            _raise(e)
        self._h = h

    def clone(self, precision: int | None = None) -> "Ilu0":
        """A factor object on the same pattern, without analysing it again (``fv_ilu0_clone``):
        ``precision`` 32 / 64 (default: this one's) gives a factor ready for :meth:`refactor`;
        0 a structure-only template to clone later factors from."""
        prec = self._precision if precision is None else int(precision)
        obj = Ilu0.__new__(Ilu0)
        obj._indptr, obj._indices = self._indptr, self._indices
        obj._n, obj._b = self._n, self._b
        obj._precision = prec
        obj._dtype = torch.float64 if prec == 64 else torch.float32
        obj._nvals = self._nvals
        h = ctypes.c_void_p()
        check(lib().fv_ilu0_clone(self._h, prec, _stream(), ctypes.byref(h)))
        obj._h = h
        return obj

    @property
    def nnz(self) -> int:
        return self._nvals

    @property
    def n(self) -> int:
        return self._n * self._b

    def refactor(self, values) -> None:
        v = torch.as_tensor(values)
        if v.numel() != self._nvals:
            raise ValueError(f"expected {self._nvals} values for this pattern, got {v.numel()}.")
        is64 = v.dtype == torch.float64
        v = v.to("cuda").contiguous()
        if self._precision == 64 and not is64:
            v = v.to(torch.float64)
        if self._precision == 32 and v.dtype not in (torch.float32, torch.float64):
            v = v.to(torch.float64)
        try:
            check(lib().fv_ilu0_factor(self._h, ptr(v), int(v.dtype == torch.float64), _stream()))
        except FvError as e:
            _raise(e)

    def factor_values(self) -> torch.Tensor:
        out = torch.empty(self._nvals, dtype=self._dtype, device="cuda")
        check(lib().fv_ilu0_factor_values(self._h, ptr(out), _stream()))
        return out

    def solve(self, rhs, transpose: bool = False, out: torch.Tensor | None = None) -> torch.Tensor:
        r = torch.as_tensor(rhs).to("cuda", dtype=self._dtype).contiguous()
        x = torch.empty_like(r) if out is None else out
        check(lib().fv_ilu0_apply(self._h, ptr(r), ptr(x), int(bool(transpose)), _stream()))
        return x

    @property
    def pivots(self) -> torch.Tensor:
        f = self.factor_values().reshape(-1, self._b, self._b)
        diag_blocks = []
        ip, ix = self._indptr, self._indices
        for i in range(self._n):
            q = ip[i] + int(np.searchsorted(ix[ip[i]:ip[i + 1]], i))
            diag_blocks.append(q)
        d = f[torch.as_tensor(diag_blocks, device="cuda")]
        return torch.diagonal(d, dim1=1, dim2=2).reshape(-1)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().fv_ilu0_destroy(h)
            except Exception:
                pass
