"""Aggregation multigrid V-cycle with ILU(0) smoothing, fp32, on the GPU.

The reference's ILU-smoothed V-cycle (``IluSmoothedInverse``, ``aquaflux/solve/ilu_inverse.py:
160-308``: ILU(0) pre-/post-smoothing sweeps ``x <- x + M^-1 (b - A x)``, restriction ``P^T``,
coarse correction, prolongation ``P``) over an aggregation hierarchy
(``aquaflux/solve/multigrid.py:1011-1245``), restated for the GPU: cells are aggregated once per
pattern on the host (``fv_aggregate``), every level's operator is the Galerkin product of the
unsmoothed aggregation (formed on the GPU by ordered block sums), and the smoothing, residuals,
restriction and prolongation all run in fp32 on the device.  The coarsest level is smoothed by
ILU(0) sweeps instead of the reference's dense inverse (the 2M-cell hierarchy's coarsest level is
too large for a dense factor).  Vectors inside the hierarchy are cell-major.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from ._lib import check, lib, ptr
from .ilu0 import Ilu0


def _stream() -> int:
    return int(torch.cuda.current_stream().cuda_stream)


class _Level:
    def __init__(self, n, b, indptr, indices):
        self.n, self.b = n, b
        self.indptr = np.ascontiguousarray(indptr, dtype=np.int32)
        self.indices = np.ascontiguousarray(indices, dtype=np.int32)
        self.nnzb = int(self.indptr[-1])
        self.d_indptr = torch.tensor(self.indptr, device="cuda")
        self.d_indices = torch.tensor(self.indices, device="cuda")
        self.values = torch.zeros(self.nnzb * b * b, dtype=torch.float32, device="cuda")
        self.ilu = Ilu0.__new__(Ilu0)
        self.ilu._setup(self.indptr, self.indices, b, 32)
        self.x = torch.zeros(n * b, dtype=torch.float32, device="cuda")
        self.r = torch.zeros_like(self.x)
        self.t = torch.zeros_like(self.x)
        self.coarse = None  # transfer data to the next level

    def spmv(self, x, y):
        check(lib().fv_bsr_spmv_f32(self.n, self.b, ptr(self.d_indptr), ptr(self.d_indices),
                                    ptr(self.values), ptr(x), ptr(y), 0, _stream()))


class AmgHierarchy:
    """Aggregation hierarchy on a fixed block pattern; ``refresh(values)`` re-forms every level."""

    def __init__(self, n, b, indptr, indices, *, min_cells: int = 4000, max_levels: int = 10,
                 sweeps: int = 1, coarse_sweeps: int = 4):
        self.b, self.sweeps, self.coarse_sweeps = b, sweeps, coarse_sweeps
        self.levels = [_Level(n, b, indptr, indices)]
        while self.levels[-1].n > min_cells and len(self.levels) < max_levels:
            fine = self.levels[-1]
            agg = np.empty(fine.n, dtype=np.int32)
            na = ctypes.c_int(0)
            check(lib().fv_aggregate(fine.n, ptr(fine.indptr), ptr(fine.indices), ptr(agg),
                                     ctypes.byref(na)))
            na = int(na.value)
            if na >= fine.n * 0.9:  # aggregation stalled
                break
            members = np.argsort(agg, kind="stable").astype(np.int32)
            mptr = np.zeros(na + 1, dtype=np.int32)
            np.cumsum(np.bincount(agg, minlength=na), out=mptr[1:])
            rows = np.repeat(np.arange(fine.n, dtype=np.int64), np.diff(fine.indptr))
            key = agg[rows].astype(np.int64) * na + agg[fine.indices]
            ukey, qmap = np.unique(key, return_inverse=True)
            cip = np.zeros(na + 1, dtype=np.int64)
            np.cumsum(np.bincount((ukey // na).astype(np.int64), minlength=na), out=cip[1:])
            cix = (ukey % na).astype(np.int32)
            glist = np.argsort(qmap, kind="stable").astype(np.int64)
            gptr = np.zeros(ukey.size + 1, dtype=np.int64)
            np.cumsum(np.bincount(qmap, minlength=ukey.size), out=gptr[1:])
            fine.coarse = {
                "agg": torch.tensor(agg, device="cuda"),
                "mptr": torch.tensor(mptr, device="cuda"),
                "mlist": torch.tensor(members, device="cuda"),
                "gptr": torch.tensor(gptr, device="cuda"),
                "glist": torch.tensor(glist, device="cuda"),
                "n_coarse_blocks": int(ukey.size),
            }
            self.levels.append(_Level(na, b, cip.astype(np.int32), cix))

    @property
    def sizes(self):
        return [lv.n for lv in self.levels]

    def refresh(self, fine_values: torch.Tensor) -> None:
        """Re-form every level from the fine operator's block values (fp64 or fp32, device)."""
        lv0 = self.levels[0]
        lv0.values.copy_(fine_values)
        lv0.ilu.refactor(fine_values)
        for fine, coarse in zip(self.levels[:-1], self.levels[1:]):
            t = fine.coarse
            check(lib().fv_galerkin_f32(t["n_coarse_blocks"], self.b, ptr(t["gptr"]),
                                        ptr(t["glist"]), ptr(fine.values), 0,
                                        ptr(coarse.values), _stream()))
            coarse.ilu.refactor(coarse.values)

    def _smooth(self, lv, b_vec, x, sweeps, from_zero):
        if from_zero:
            lv.ilu.solve(b_vec, out=x)
            sweeps -= 1
        for _ in range(sweeps):
            lv.spmv(x, lv.t)
            torch.sub(b_vec, lv.t, out=lv.r)
            lv.ilu.solve(lv.r, out=lv.t)
            x.add_(lv.t)

    def vcycle(self, level: int, b_vec: torch.Tensor) -> torch.Tensor:
        lv = self.levels[level]
        x = lv.x
        if level == len(self.levels) - 1:
            self._smooth(lv, b_vec, x, self.coarse_sweeps, True)
            return x
        self._smooth(lv, b_vec, x, self.sweeps, True)
        lv.spmv(x, lv.t)
        torch.sub(b_vec, lv.t, out=lv.r)
        coarse = self.levels[level + 1]
        t = lv.coarse
        bc = torch.empty(coarse.n * self.b, dtype=torch.float32, device="cuda")
        check(lib().fv_restrict_f32(coarse.n, self.b, ptr(t["mptr"]), ptr(t["mlist"]), ptr(lv.r),
                                    ptr(bc), _stream()))
        xc = self.vcycle(level + 1, bc)
        check(lib().fv_prolong_add_f32(lv.n, self.b, ptr(t["agg"]), ptr(xc), ptr(x), _stream()))
        self._smooth(lv, b_vec, x, self.sweeps, False)
        return x


class AmgPreconditioner:
    """``M ~= J^-1``: one fp32 aggregation V-cycle with ILU(0) smoothing of the materialised block
    Jacobian (field-major fp64 vectors in and out)."""

    def __init__(self, jac, **kw):
        self.jac = jac
        self.h = AmgHierarchy(jac.n, jac.b, jac.indptr, jac.indices, **kw)
        self._b = torch.empty(jac.n * jac.b, dtype=torch.float32, device="cuda")

    def refresh(self, state: torch.Tensor) -> None:
        self.h.refresh(self.jac.materialize(state))

    def apply(self, r: torch.Tensor) -> torch.Tensor:
        n, b = self.jac.n, self.jac.b
        self._b.copy_(r.view(b, n).t().reshape(-1))
        x = self.h.vcycle(0, self._b)
        return x.view(n, b).t().reshape(-1).to(torch.float64)
