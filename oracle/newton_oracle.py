"""Newton's method on the CPU oracle with an exact sparse Jacobian and a sparse direct solve --
test infrastructure only: the independent FP64 root the GPU Newton solve is checked against, and
the CPU Newton-solve time reported beside the GPU's (never on the product path).

The method is the reference's ``ImplicitNewtonSolver`` (``aquaflux/solve/implicit.py:767-864``):
Newton steps to ``||R|| <= atol + rtol ||R_0||`` (``within_tolerance``,
``aquaflux/solve/forward_step.py:352``; 1e-12, 1e-10) with the backtracking line search of
``implicit.py:270-455`` (largest ``alpha`` in 1, 1/2, ... that lowers ``||R||``).  Only the linear
solve differs: the reference's inexact GMRES (``implicit.py:50``) is replaced by an exact sparse LU
(SuperLU through scipy) of the exact Jacobian, so the root does not depend on any Krylov iterate.

The Jacobian is recovered from reverse-mode products of the oracle (``Oracle.vjp``), one per
(colour, field): the rows of one colour share no column of the reach-3 cell pattern (the exact
Jacobian's reach for these residuals, ``aquaflux/solve/sparse_jacobian.py:358-360``), so
``u^T J`` with ``u`` the indicator of those rows holds each of them separately.  The colouring is
a plain greedy distance-2 colouring (any valid colouring gives the same Jacobian).
"""
from __future__ import annotations

import math
import time

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla
import torch


def cell_stencil(owner, neighbour, n: int, reach: int = 3) -> sp.csr_matrix:
    """Cells within graph distance ``reach`` of each cell (diagonal included), 0/1 CSR."""
    own = np.asarray(owner)
    nb = np.asarray(neighbour)
    keep = nb >= 0
    own, nb = own[keep], nb[keep]
    rows = np.concatenate([own, nb, np.arange(n)])
    cols = np.concatenate([nb, own, np.arange(n)])
    adj = sp.coo_matrix((np.ones(rows.size), (rows, cols)), shape=(n, n)).tocsr()
    adj.data[:] = 1.0
    pat = adj
    for _ in range(reach - 1):
        pat = (pat @ adj).tocsr()
        pat.data[:] = 1.0
    pat.sort_indices()
    return pat


def greedy_colouring(pat: sp.csr_matrix) -> np.ndarray:
    """Colours such that two cells sharing a column of ``pat`` (symmetric) differ."""
    conflict = (pat.T @ pat).tocsr()
    n = pat.shape[0]
    colour = np.full(n, -1, dtype=np.int64)
    ip, ix = conflict.indptr, conflict.indices
    for c in range(n):
        used = colour[ix[ip[c]:ip[c + 1]]]
        taken = np.zeros(used.size + 2, dtype=bool)
        taken[used[(used >= 0) & (used < taken.size)]] = True
        colour[c] = int(np.argmin(taken))
    return colour


class OracleJacobian:
    """Exact sparse Jacobian of an :class:`oracle.fv_oracle.Oracle` residual (field-major
    unknowns ``q * n + c``)."""

    def __init__(self, orc, owner, neighbour, n_cells: int, n_fields: int, reach: int = 3):
        self.orc = orc
        self.n, self.b = n_cells, n_fields
        self.pat = cell_stencil(owner, neighbour, n_cells, reach)
        self.colour = greedy_colouring(self.pat)
        self.n_colours = int(self.colour.max()) + 1
        deg = np.diff(self.pat.indptr)
        self._rows_cell = np.repeat(np.arange(n_cells), deg)
        self._cols_cell = self.pat.indices

    def matrix(self, x) -> sp.csc_matrix:
        n, b = self.n, self.b
        rows, cols, vals = [], [], []
        for k in range(self.n_colours):
            sel = self.colour[self._rows_cell] == k  # pattern entries of this colour's rows
            rc, cc = self._rows_cell[sel], self._cols_cell[sel]
            cells = np.flatnonzero(self.colour == k)
            for q in range(b):
                u = np.zeros(b * n)
                u[q * n + cells] = 1.0
                g = self.orc.vjp(x, u).numpy()
                for p in range(b):
                    rows.append(q * n + rc)
                    cols.append(p * n + cc)
                    vals.append(g[p * n + cc])
        J = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                          shape=(b * n, b * n))
        return J.tocsc()


def newton(orc, jac: OracleJacobian, x0, *, rtol: float = 1e-10, atol: float = 1e-12,
           max_steps: int = 40, line_search_steps: int = 10, min_steps: int = 0) -> dict:
    """Damped Newton with exact sparse LU solves; returns the state, the residual norms, the step
    count and the seconds spent.  ``min_steps`` forces that many steps even when the start already
    meets the tolerance (to refine a root another solver produced)."""
    t0 = time.perf_counter()
    x = np.array(x0, dtype=np.float64)
    r = orc.residual(torch.as_tensor(x)).numpy()
    norms = [float(np.linalg.norm(r))]
    target = atol + rtol * norms[0]
    steps = 0
    while (norms[-1] > target or steps < min_steps) and steps < max_steps:
        J = jac.matrix(x)
        dx = spla.spsolve(J, -r)
        alpha, best = 1.0, None
        for _ in range(line_search_steps + 1):
            cand = x + alpha * dx
            rc = orc.residual(torch.as_tensor(cand)).numpy()
            nc = float(np.linalg.norm(rc))
            if math.isfinite(nc):
                if best is None or nc < best[2]:
                    best = (cand, rc, nc)
                if nc < norms[-1]:
                    break
            alpha *= 0.5
        if best is None:
            break
        x, r, nrm = best
        steps += 1
        if nrm >= norms[-1] and steps > min_steps:
            norms.append(nrm)
            break
        norms.append(nrm)
    return {"state": x, "residual_norms": norms, "steps": steps,
            "converged": norms[-1] <= target, "seconds": time.perf_counter() - t0}
