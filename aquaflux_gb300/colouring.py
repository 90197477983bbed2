"""Block-stencil colouring and the compressed Jacobian probe plan.

Mirrors ``block_stencil_colouring`` (``aquaflux/solve/sparse_jacobian.py:338-402``): the reach-r
cell pattern is the r-th power of the cell adjacency (self loops included), two columns conflict
when they share a row of that pattern (``P^T P``), and the conflict graph is coloured by the
saturation-degree greedy heuristic.  The sparse products are formed with the same scipy
operations as the reference, so the conflict graph -- and with it the neighbour order the
colouring's tie-breaks depend on -- is identical; the colouring itself runs in the C library
(``fv_saturation_colouring``), which restates the reference's bucket-queue algorithm.
"""
from __future__ import annotations

import ctypes
import dataclasses

import numpy as np
import scipy.sparse as sp

from ._lib import check, lib, ptr


@dataclasses.dataclass
class BlockColouring:
    n_cells: int
    reach: int
    colour: np.ndarray  # (n_cells,) int
    n_colours: int
    pattern_rows: np.ndarray  # block pattern (cell rows / cols), COO order of the pattern
    pattern_cols: np.ndarray


def _check_graph(n: int, owner: np.ndarray, nb: np.ndarray) -> None:
    if owner.shape != nb.shape or owner.ndim != 1:
        raise ValueError("block_stencil_colouring: owner and neighbour must be 1-D and equal length")
    if owner.size and (owner.min() < 0 or owner.max() >= n or nb.min() < 0 or nb.max() >= n):
        raise ValueError("block_stencil_colouring: cell index out of range")


def stencil_pattern(owner, nb, n: int, reach: int) -> sp.csr_matrix:
    """Cells within graph distance ``reach`` (diagonal included), as a 0/1 CSR matrix."""
    owner, nb = np.asarray(owner), np.asarray(nb)
    ones = np.ones(2 * owner.size + n)
    rows = np.concatenate([owner, nb, np.arange(n)])
    cols = np.concatenate([nb, owner, np.arange(n)])
    adj = sp.coo_matrix((ones, (rows, cols)), shape=(n, n)).tocsr()
    adj.data[:] = 1.0
    pat = adj
    for _ in range(reach - 1):
        pat = pat @ adj
        pat.data[:] = 1.0
    return pat


def cell_pattern(owner, nb, n: int) -> tuple[np.ndarray, np.ndarray]:
    """The reach-1 pattern (``stencil_pattern(.., 1)``) as sorted int32 CSR arrays, built by
    ``fv_cell_pattern``."""
    owner = np.ascontiguousarray(owner, dtype=np.int32)
    nb = np.ascontiguousarray(nb, dtype=np.int32)
    indptr = np.empty(n + 1, dtype=np.int32)
    indices = np.empty(n + 2 * owner.size, dtype=np.int32)
    check(lib().fv_cell_pattern(n, owner.size, ptr(owner), ptr(nb), ptr(indptr), ptr(indices)))
    nnz = int(indptr[-1])
    return indptr, (indices if nnz == indices.size else indices[:nnz].copy())


def saturation_colouring(conflict: sp.csr_matrix) -> np.ndarray:
    n = conflict.shape[0]
    ip = np.ascontiguousarray(conflict.indptr, dtype=np.int32)
    ix = np.ascontiguousarray(conflict.indices, dtype=np.int32)
    colour = np.empty(n, dtype=np.int32)
    nc = ctypes.c_int(0)
    check(lib().fv_saturation_colouring(n, ptr(ip), ptr(ix), ptr(colour), ctypes.byref(nc)))
    return colour.astype(np.int64)


def block_stencil_colouring(owner, nb, n: int, reach: int) -> BlockColouring:
    """Colour the cells so that columns sharing a row of the reach-``reach`` pattern differ.

    ``owner`` / ``nb`` are the interior-face cell pairs (the cell graph's edges).
    """
    owner, nb = np.asarray(owner), np.asarray(nb)
    _check_graph(n, owner, nb)
    if reach < 1:
        raise ValueError(f"block_stencil_colouring: reach must be >= 1, got {reach}.")
    pat = stencil_pattern(owner, nb, n, reach)
    conflict = (pat.T @ pat).tocsr()
    conflict.data[:] = 1.0
    colour = saturation_colouring(conflict)
    coo = pat.tocoo()
    return BlockColouring(n, reach, colour, int(colour.max()) + 1 if n else 0, coo.row, coo.col)
