"""Aggregation multigrid V-cycle with ILU(0) smoothing, fp32, on the GPU.

The reference's ILU-smoothed V-cycle (``IluSmoothedInverse``, ``aquaflux/solve/ilu_inverse.py:
160-308``: ILU(0) pre-/post-smoothing sweeps ``x <- x + M^-1 (b - A x)``, restriction ``P^T``,
coarse correction, prolongation ``P``) over an aggregation hierarchy
(``aquaflux/solve/multigrid.py:1011-1245``), restated for the GPU: cells are aggregated once per
pattern on the host (``fv_aggregate``), every level's operator is the Galerkin product of the
unsmoothed aggregation (formed on the GPU by ordered block sums), and the smoothing, residuals,
restriction and prolongation all run on the device, in fp32 (the mixed-precision preconditioner)
or fp64.  The coarsest level is smoothed by
ILU(0) sweeps instead of the reference's dense inverse (the 2M-cell hierarchy's coarsest level is
too large for a dense factor).  Coarse aggregates are numbered colour by colour, so that the coarse
levels' ILU(0) sweeps run in a handful of level sets.  Vectors inside the hierarchy are
cell-major.
"""
from __future__ import annotations

import ctypes
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import torch

from ._lib import FV_ERR_ZERO_PIVOT, FvError, check, lib, ptr
from .ilu0 import Ilu0


def _stream() -> int:
    return int(torch.cuda.current_stream().cuda_stream)


class _Level:
    """One level's operator storage, smoother and work vectors.  ``kept``: the connectivity-only
    part of this level (device pattern, a structure-only ILU(0) template) from an earlier
    hierarchy on the same pattern, reused as is; an empty dict is filled for later ones."""

    def __init__(self, n, b, indptr, indices, precision, kept: dict | None = None):
        self.n, self.b = n, b
        self.sfx = "f32" if precision == 32 else "f64"
        dtype = torch.float32 if precision == 32 else torch.float64
        self.indptr = np.ascontiguousarray(indptr, dtype=np.int32)
        self.indices = np.ascontiguousarray(indices, dtype=np.int32)
        self.nnzb = int(self.indptr[-1])
        if kept:
            self.d_indptr, self.d_indices = kept["d_indptr"], kept["d_indices"]
            self.ilu = kept["ilu"].clone(precision)
        else:
            self.d_indptr = torch.tensor(self.indptr, device="cuda")
            self.d_indices = torch.tensor(self.indices, device="cuda")
            self.ilu = Ilu0.__new__(Ilu0)
            self.ilu._setup(self.indptr, self.indices, b, precision)
            if kept is not None:
                kept.update(d_indptr=self.d_indptr, d_indices=self.d_indices,
                            ilu=self.ilu.clone(0))
        self.values = torch.zeros(self.nnzb * b * b, dtype=dtype, device="cuda")
        self.x = torch.zeros(n * b, dtype=dtype, device="cuda")
        self.r = torch.zeros_like(self.x)
        self.t = torch.zeros_like(self.x)
        self.rhs = torch.zeros_like(self.x)  # right-hand side when this is a coarse level
        self.coarse = None  # transfer data to the next level
        # the transpose (map and transposed blocks), built on the first transposed product and
        # re-formed with the values after every refresh
        self._tmap = None
        self._tvals = None

    def transpose_values(self) -> None:
        """Re-form the transposed blocks from ``values`` (nothing before a transposed product)."""
        if self._tvals is not None:
            check(lib().fv_bsr_transpose_blocks(self.nnzb, self.b, ptr(self._tmap[2]),
                                                ptr(self.values), ptr(self._tvals),
                                                int(self.sfx == "f64"), _stream()))

    def spmv(self, x, y, transpose: bool = False):
        if not transpose:
            check(getattr(lib(), "fv_bsr_spmv_" + self.sfx)(
                self.n, self.b, ptr(self.d_indptr), ptr(self.d_indices), ptr(self.values), ptr(x),
                ptr(y), 0, _stream()))
            return
        if self._tmap is None:
            tp = np.empty(self.n + 1, dtype=np.int32)
            ti = np.empty(self.nnzb, dtype=np.int32)
            tb = np.empty(self.nnzb, dtype=np.int32)
            check(lib().fv_bsr_transpose_map(self.n, ptr(self.indptr), ptr(self.indices), ptr(tp),
                                             ptr(ti), ptr(tb)))
            self._tmap = [torch.tensor(a, device="cuda") for a in (tp, ti, tb)]
            self._tvals = torch.empty_like(self.values)
            self.transpose_values()
        # A^T x as the forward product on A^T's pattern and transposed blocks: the products of
        # the mapped transposed kernel in the same order, read row-wise
        tp, ti, _ = self._tmap
        check(getattr(lib(), "fv_bsr_spmv_" + self.sfx)(
            self.n, self.b, ptr(tp), ptr(ti), ptr(self._tvals), ptr(x), ptr(y), 0, _stream()))


def plan_hierarchy(n, indptr, indices, *, min_cells: int = 4000, max_levels: int = 10,
                   coarse_order: str = "colour") -> list[dict]:
    """Host plan of the aggregation hierarchy over a cell graph (sorted CSR with self loops).

    One entry per coarsening: ``agg`` (fine cell -> aggregate), ``mptr``/``mlist`` (members of
    each aggregate), the coarse pattern ``indptr``/``indices`` and, per coarse block, the ordered
    list of fine blocks summed into it (``gptr``/``glist``).  With ``coarse_order="colour"`` the
    aggregates are numbered colour by colour (saturation colouring of the aggregate graph): rows of
    one colour are independent, so the coarse ILU(0) sweeps need as many level sets as there are
    colours instead of hundreds.
    """
    ip = np.ascontiguousarray(indptr, dtype=np.int32)
    ix = np.ascontiguousarray(indices, dtype=np.int32)
    plan = []
    while n > min_cells and len(plan) + 1 < max_levels:
        agg = np.empty(n, dtype=np.int32)
        na = ctypes.c_int(0)
        check(lib().fv_aggregate(n, ptr(ip), ptr(ix), ptr(agg), ctypes.byref(na)))
        na = int(na.value)
        if na >= n * 0.9:  # aggregation stalled
            break
        if coarse_order == "colour":
            col = np.empty(na, dtype=np.int32)
            nco = ctypes.c_int(0)
            check(lib().fv_colour_aggregates(n, ptr(ip), ptr(ix), ptr(agg), na, ptr(col),
                                             ctypes.byref(nco)))
            order = np.concatenate([np.flatnonzero(col == c) for c in range(nco.value)])
            newid = np.empty(na, dtype=np.int32)
            newid[order] = np.arange(na, dtype=np.int32)
            agg = newid[agg]
        step = _coarsen(n, ip, ix, agg, na)
        plan.append(step)
        cip, cix = step["indptr"], step["indices"]
        n, ip, ix = na, cip, cix
    return plan


def _coarsen(n, ip, ix, agg, na, lists: bool = True) -> dict:
    """One coarsening step (``fv_coarsen``): members, coarse pattern, ordered fine-block lists."""
    nnz = int(ip[-1])
    mptr = np.empty(na + 1, dtype=np.int32)
    mlist = np.empty(n, dtype=np.int32)
    cip = np.empty(na + 1, dtype=np.int32)
    cix = np.empty(nnz, dtype=np.int32)
    gptr = np.empty(nnz + 1, dtype=np.int64) if lists else None
    glist = np.empty(nnz, dtype=np.int64) if lists else None
    ncb = ctypes.c_long(0)
    agg = np.ascontiguousarray(agg, dtype=np.int32)
    check(lib().fv_coarsen(n, ptr(ip), ptr(ix), ptr(agg), na, ptr(mptr), ptr(mlist), ptr(cip),
                           ptr(cix), ptr(gptr), ptr(glist), ctypes.byref(ncb)))
    ncb = int(ncb.value)
    return {"n_coarse": na, "agg": agg, "mptr": mptr, "mlist": mlist, "indptr": cip,
            "indices": cix[:ncb], "gptr": gptr[:ncb + 1] if lists else None, "glist": glist}


class AmgHierarchy:
    """Aggregation hierarchy on a fixed block pattern; ``refresh(values)`` re-forms every level.

    The coarsest level is smoothed by ``coarse_sweeps`` ILU(0) sweeps (``coarse_solve="ilu"``,
    default), or solved exactly by a dense inverse (``"dense"``, the reference's coarsest-level
    inverse; ``"auto"``: dense when it has at most ``dense_max`` unknowns).  The inverse is formed
    in the hierarchy's precision by LU with partial pivoting (cuSOLVER) at every refresh and
    applied as one dense matrix-vector product.  On the 128^3 SST channel (coarsest level 303
    cells) the dense solve makes a V-cycle 0.4 ms cheaper but the fp32 Newton solve takes one
    more step (9 / 99 Krylov iterations instead of 8 / 95), and the fp64 inverse costs ~40 ms
    per refresh, so the sweeps stay the default.

    The host plan of the coarse levels runs on a worker thread while the fine level's ILU(0)
    structures are built.
    """

    def __init__(self, n, b, indptr, indices, *, min_cells: int = 4000, max_levels: int = 10,
                 sweeps: int = 1, coarse_sweeps: int = 4, coarse_order: str = "colour",
                 precision: int = 32, coarse_solve: str = "ilu", dense_max: int = 4096,
                 plan=None, kept: dict | None = None):
        if precision not in (32, 64):
            raise ValueError(f"precision must be 32 or 64, got {precision}")
        if coarse_solve not in ("auto", "dense", "ilu"):
            raise ValueError(f"coarse_solve must be 'auto', 'dense' or 'ilu', got {coarse_solve!r}")
        self.b, self.sweeps, self.coarse_sweeps = b, sweeps, coarse_sweeps
        self.precision = precision
        self.sfx = "f32" if precision == 32 else "f64"
        # kept["levels"][l]: level l's connectivity-only device structures, shared by every
        # hierarchy on this pattern (filled by the first)
        klv = None if kept is None else kept.setdefault("levels", [])
        kl = (lambda i: None if klv is None else
              (klv[i] if i < len(klv) else klv.append({}) or klv[i]))
        if plan is None:
            with ThreadPoolExecutor(1) as pool:
                plan = pool.submit(plan_hierarchy, n, indptr, indices, min_cells=min_cells,
                                   max_levels=max_levels, coarse_order=coarse_order)
                self.levels = [_Level(n, b, indptr, indices, precision, kl(0))]
                plan = plan.result()
        else:  # a given plan (a list, or the future of one still being made)
            self.levels = [_Level(n, b, indptr, indices, precision, kl(0))]
            plan = plan.result() if hasattr(plan, "result") else plan
        for i, step in enumerate(plan):
            fine = self.levels[-1]
            kf = kl(i)
            if kf is not None and "coarse" in kf:
                fine.coarse = dict(kf["coarse"])
            else:
                fine.coarse = {k: torch.tensor(step[k], device="cuda")
                               for k in ("agg", "mptr", "mlist", "gptr", "glist")}
                fine.coarse["n_coarse_blocks"] = int(step["gptr"].size - 1)
                if kf is not None:
                    kf["coarse"] = dict(fine.coarse)
            self.levels.append(_Level(step["n_coarse"], b, step["indptr"], step["indices"],
                                      precision, kl(i + 1)))
        last = self.levels[-1]
        nd = last.n * b
        self.dense = None
        if len(self.levels) > 1 and (coarse_solve == "dense"
                                     or (coarse_solve == "auto" and nd <= dense_max)):
            # flat position of every coarse block entry in the dense (nd x nd) row-major matrix
            rows = np.repeat(np.arange(last.n, dtype=np.int64), np.diff(last.indptr))
            cols = last.indices.astype(np.int64)
            r = np.arange(b, dtype=np.int64)
            pos = (((rows[:, None, None] * b + r[None, :, None]) * nd)
                   + cols[:, None, None] * b + r[None, None, :])
            self.dense = {"pos": torch.tensor(pos.reshape(-1), device="cuda"),
                          "a": torch.zeros(nd, nd, dtype=last.values.dtype, device="cuda"),
                          "inv": torch.zeros(nd, nd, dtype=last.values.dtype, device="cuda")}

    @property
    def coarse_solve(self) -> str:
        return "dense" if self.dense is not None else "ilu"

    def _invert_coarsest(self) -> None:
        d, lv = self.dense, self.levels[-1]
        d["a"].zero_()
        d["a"].view(-1).index_copy_(0, d["pos"], lv.values)
        inv, info = torch.linalg.inv_ex(d["a"])
        if int(info) != 0:
            raise FvError(FV_ERR_ZERO_PIVOT,
                          f"the coarsest AMG operator ({lv.n} cells) is singular: LU met an "
                          f"exactly zero pivot at column {int(info) - 1}", int(info) - 1)
        d["inv"].copy_(inv)

    @property
    def sizes(self):
        return [lv.n for lv in self.levels]

    def refresh(self, fine_values: torch.Tensor, bmap: torch.Tensor | None = None) -> None:
        """Re-form every level from the fine operator's block values (fp64 or fp32, device);
        with ``bmap`` the hierarchy's fine block q is block ``bmap[q]`` of ``fine_values``."""
        lv0 = self.levels[0]
        if bmap is not None:
            check(lib().fv_gather_blocks(lv0.nnzb, self.b, ptr(bmap), ptr(fine_values),
                                         int(fine_values.dtype == torch.float64),
                                         ptr(lv0.values), int(self.precision == 64), _stream()))
        elif self.precision == 64 and fine_values.dtype == torch.float64:
            lv0.values = fine_values  # the fine operator itself (no copy)
        else:
            lv0.values.copy_(fine_values)
        lv0.ilu.refactor(lv0.values)
        galerkin = getattr(lib(), "fv_galerkin_" + self.sfx)
        for fine, coarse in zip(self.levels[:-1], self.levels[1:]):
            t = fine.coarse
            check(galerkin(t["n_coarse_blocks"], self.b, ptr(t["gptr"]), ptr(t["glist"]),
                           ptr(fine.values), int(fine.values.dtype == torch.float64),
                           ptr(coarse.values), _stream()))
            if coarse is self.levels[-1] and self.dense is not None:
                self._invert_coarsest()
            else:
                coarse.ilu.refactor(coarse.values)
        for lv in self.levels:
            lv.transpose_values()

    def _smooth(self, lv, b_vec, x, sweeps, from_zero, transpose=False):
        if from_zero:
            lv.ilu.solve(b_vec, transpose=transpose, out=x)
            sweeps -= 1
        for _ in range(sweeps):
            lv.spmv(x, lv.t, transpose)
            torch.sub(b_vec, lv.t, out=lv.r)
            lv.ilu.solve(lv.r, transpose=transpose, out=lv.t)
            x.add_(lv.t)

    def vcycle(self, level: int, b_vec: torch.Tensor, transpose: bool = False) -> torch.Tensor:
        """One V-cycle from a zero guess; ``transpose`` gives its exact transpose, the same cycle
        on ``A^T`` with transposed ILU(0) smoothers (the pre- and post-smoother coincide and
        ``R = P^T``), as the reference's V-cycle transpose (``ilu_inverse.py:275-308``)."""
        lv = self.levels[level]
        x = lv.x
        if level == len(self.levels) - 1:
            if self.dense is not None:
                inv = self.dense["inv"]
                torch.mv(inv.t() if transpose else inv, b_vec, out=x)
            else:
                self._smooth(lv, b_vec, x, self.coarse_sweeps, True, transpose)
            return x
        self._smooth(lv, b_vec, x, self.sweeps, True, transpose)
        lv.spmv(x, lv.t, transpose)
        torch.sub(b_vec, lv.t, out=lv.r)
        coarse = self.levels[level + 1]
        t = lv.coarse
        bc = coarse.rhs
        check(getattr(lib(), "fv_restrict_" + self.sfx)(
            coarse.n, self.b, ptr(t["mptr"]), ptr(t["mlist"]), ptr(lv.r), ptr(bc), _stream()))
        xc = self.vcycle(level + 1, bc, transpose)
        check(getattr(lib(), "fv_prolong_add_" + self.sfx)(
            lv.n, self.b, ptr(t["agg"]), ptr(xc), ptr(x), _stream()))
        self._smooth(lv, b_vec, x, self.sweeps, False, transpose)
        return x


class AmgPreconditioner:
    """``M ~= J^-1``: one aggregation V-cycle with ILU(0) smoothing of the materialised block
    Jacobian, fp32 (default) or fp64 throughout (field-major fp64 vectors in and out).

    ``fine_order="natural"`` keeps the operator's own cell order for the fine ILU(0) smoother;
    ``"colour"`` numbers the fine cells colour by colour (a first-fit colouring of the cell graph:
    a few colours on a hexahedral mesh), so that the fine sweeps run in a few wide level sets
    instead of ~3N narrow ones -- much cheaper per cycle, a weaker smoother.  ``"auto"`` (default)
    takes the coloured order in 3D, where it wins (128^3 SST channel: 95 instead of 72 Krylov
    iterations, each V-cycle ~4x cheaper), and the natural order in 2D, where the coloured smoother
    stalls on laminar saddle-point systems.  Coarse levels are always colour-numbered.

    ``graph=True`` (default) replays the V-cycle as one CUDA graph, captured on the second
    application after each re-form of the fine operator's storage: the coarse levels are
    hundreds of launches of a few microseconds each, which the host would otherwise issue one by
    one.  The forward and the transposed cycle (the IFT adjoint's) keep a graph each.
    """

    def __init__(self, jac, precision: int = 32, *, fine_order: str = "auto", shift=None,
                 equilibrate: bool = False, graph: bool = True, **kw):
        from .solve import ShiftedCellMajorOperator

        self.jac = jac
        n, b = jac.n, jac.b
        self._perm = self._bmap = None
        indptr, indices = jac.indptr, jac.indices
        if fine_order == "auto":
            fine_order = "colour" if jac.case.dim == 3 else "natural"
        self.fine_order = fine_order
        # connectivity-only products, built once per case (FlowCase.pattern_plan)
        cache = getattr(jac.case, "pattern_plan", None)
        plan_key = tuple(sorted((k, kw[k]) for k in ("min_cells", "max_levels", "coarse_order")
                                if k in kw))
        cached = (lambda key, build: cache((key, jac.reach) + plan_key, build)
                  ) if cache is not None else (lambda key, build: build())
        if fine_order == "colour":
            def colour_order():
                col = np.empty(n, dtype=np.int32)
                nco = ctypes.c_int(0)
                check(lib().fv_greedy_colouring(n, ptr(indptr), ptr(indices), ptr(col),
                                                ctypes.byref(nco)))
                perm = np.concatenate([np.flatnonzero(col == c)
                                       for c in range(nco.value)]).astype(np.int32)
                pip = np.empty(n + 1, dtype=np.int32)
                pix = np.empty(int(indptr[-1]), dtype=np.int32)
                bmap = np.empty(int(indptr[-1]), dtype=np.int64)
                check(lib().fv_permute_pattern(n, ptr(indptr), ptr(indices), ptr(perm),
                                               ptr(pip), ptr(pix), ptr(bmap)))
                return perm, pip, pix, bmap, int(nco.value)

            perm, pip, pix, bmap, self.n_colours = cached("amg_fine_colour_order", colour_order)
            self._perm = torch.tensor(perm, device="cuda")
            self._bmap = torch.tensor(bmap, device="cuda")
            indptr, indices = pip, pix
        elif fine_order != "natural":
            raise ValueError(f"fine_order must be 'colour' or 'natural', got {fine_order!r}")
        self.precision = precision
        self.shift = None if shift is None else torch.as_tensor(shift, dtype=torch.float64,
                                                                device="cuda")
        self.op = (ShiftedCellMajorOperator(jac, equilibrate=equilibrate, precision=64)
                   if (shift is not None or equilibrate) else None)
        # the aggregation plan runs on a worker thread (overlapping the fine level's ILU(0)
        # structures on first use); later preconditioners on this case reuse it
        plan_kw = {k: kw[k] for k in ("min_cells", "max_levels", "coarse_order") if k in kw}

        def hierarchy_plan():
            pool = ThreadPoolExecutor(1)
            fut = pool.submit(plan_hierarchy, n, indptr, indices, **plan_kw)
            pool.shutdown(wait=False)
            return fut

        plan = cached("amg_hierarchy_plan_" + fine_order, hierarchy_plan)
        kept = (cached("amg_hierarchy_structures_" + fine_order, dict) if cache is not None
                else None)
        self.h = AmgHierarchy(n, b, indptr, indices, precision=precision, plan=plan, kept=kept,
                              **kw)
        self._f64 = int(precision == 64)
        self._b = torch.empty(n * b, dtype=self.h.levels[0].x.dtype, device="cuda")
        self.graph = bool(graph)
        # per direction (False: forward, True: transposed): the captured cycle and the fine
        # storage address it was captured on, and the address of the last eager cycle
        self._graphs: dict = {}
        self._eager_keys: dict = {}

    def _form(self, values):
        if self.op is not None:
            values, _ = self.op.assemble(values, self.shift)
        self.h.refresh(values, self._bmap)

    def refresh(self, state: torch.Tensor) -> None:
        self._form(self.jac.materialize(state))

    def reshift(self, shift) -> None:
        """New shift on the last materialised Jacobian: re-form the hierarchy without
        re-materialising (the beta-only refresh of ``amg_preconditioner.py:909-948``)."""
        from .solve import ShiftedCellMajorOperator

        if self.op is None:
            self.op = ShiftedCellMajorOperator(self.jac, equilibrate=False, precision=64)
        self.shift = None if shift is None else torch.as_tensor(shift, dtype=torch.float64,
                                                                device="cuda")
        self._form(self.jac.values)

    def apply(self, r: torch.Tensor, transpose: bool = False) -> torch.Tensor:
        n, b = self.jac.n, self.jac.b
        scale = None if self.op is None else self.op.scale
        check(lib().fv_to_cells(n, b, ptr(self._perm), ptr(scale), ptr(r), ptr(self._b),
                                self._f64, _stream()))
        x = self._vcycle(transpose)
        out = torch.empty(n * b, dtype=torch.float64, device="cuda")
        check(lib().fv_from_cells(n, b, ptr(self._perm), ptr(scale), ptr(x), self._f64, ptr(out),
                                  _stream()))
        return out

    def _vcycle(self, transpose: bool) -> torch.Tensor:
        """The V-cycle (or its transpose) on ``self._b`` into the fine level's ``x``: eager, or a
        graph replay.  Under a caller's own stream capture the cycle is recorded eagerly into that
        graph."""
        if not self.graph or torch.cuda.is_current_stream_capturing():
            return self.h.vcycle(0, self._b, transpose)
        # the graph holds the fine operator's storage address (an fp64 fine level may hold the
        # Jacobian's own tensor): re-capture when it changes, after one eager cycle that builds
        # the smoothers' (transposed) solve structures and the transposed products' maps outside
        # the capture
        key = self.h.levels[0].values.data_ptr()
        held = self._graphs.get(transpose)
        if held is None or held[1] != key:
            if self._eager_keys.get(transpose) != key:
                self._eager_keys[transpose] = key
                return self.h.vcycle(0, self._b, transpose)
            # captured on a side stream through capture_begin / capture_end: the torch.cuda.graph
            # context manager would empty the caching allocator at every capture, and the next
            # solve would then re-allocate its multi-GB bases and levels from the driver
            g = torch.cuda.CUDAGraph()
            main = torch.cuda.current_stream()
            side = torch.cuda.Stream()
            side.wait_stream(main)
            with torch.cuda.stream(side):
                g.capture_begin()
                try:
                    self.h.vcycle(0, self._b, transpose)
                finally:
                    g.capture_end()
            main.wait_stream(side)
            held = self._graphs[transpose] = (g, key)
        held[0].replay()
        return self.h.levels[0].x

    def apply_transpose(self, r: torch.Tensor) -> torch.Tensor:
        """``M^T r``: the transposed V-cycle between the same (diagonal) scalings and the same
        (orthogonal) cell permutation."""
        return self.apply(r, transpose=True)
