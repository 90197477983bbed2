"""Cell renumbering on the GPU: the cell graph and reverse Cuthill-McKee.

``ReverseCuthillMcKee.permutation`` (``aquaflux/mesh/reorder.py:147-159``) relabels the cells by
scipy's ``reverse_cuthill_mckee`` on the interior-face cell graph (``cell_adjacency_coo``,
``aquaflux/mesh/graph.py:29-56``).  Here the graph is built on the GPU (``fv_cell_graph``: sorted,
coalesced CSR) and the breadth-first sweeps run on the GPU level by level
(``fv_rcm_permutation``), giving the same permutation bit for bit.  The only host step is the seed
order, numpy's ``argsort`` of the node degrees -- the call scipy's implementation makes, so ties
between equal-degree seeds resolve as they do there.
"""
from __future__ import annotations

import numpy as np
import torch

from ._lib import check, lib, ptr


def _stream() -> int:
    return int(torch.cuda.current_stream().cuda_stream)


def cell_graph(owner, neighbour, n_cells: int) -> tuple[torch.Tensor, torch.Tensor]:
    """The symmetric cell graph of the interior faces (``neighbour >= 0``) as device CSR
    ``(indptr, indices)``, neighbours ascending, repeated pairs coalesced."""
    own = torch.as_tensor(np.asarray(owner), dtype=torch.int32)
    nb = torch.as_tensor(np.asarray(neighbour), dtype=torch.int32)
    keep = nb >= 0
    own = own[keep].to("cuda").contiguous()
    nb = nb[keep].to("cuda").contiguous()
    n_pairs = int(own.numel())
    indptr = torch.empty(n_cells + 1, dtype=torch.int32, device="cuda")
    indices = torch.empty(max(2 * n_pairs, 1), dtype=torch.int32, device="cuda")
    work = torch.empty(2 * n_cells + 2 + 2 * n_pairs, dtype=torch.int32, device="cuda")
    check(lib().fv_cell_graph(n_cells, n_pairs, ptr(own), ptr(nb), ptr(indptr), ptr(indices),
                              ptr(work), _stream()))
    nnz = int(indptr[-1])
    return indptr, indices[:nnz]


def rcm_permutation(owner, neighbour, n_cells: int) -> np.ndarray:
    """``perm[old] = new`` of reverse Cuthill-McKee on the cell graph, computed on the GPU."""
    indptr, indices = cell_graph(owner, neighbour, n_cells)
    degree = torch.diff(indptr).cpu().numpy().astype(np.int32)
    seeds = np.ascontiguousarray(np.argsort(degree), dtype=np.int64)
    perm = torch.empty(n_cells, dtype=torch.int32, device="cuda")
    work = torch.empty(3 * n_cells + 1, dtype=torch.int32, device="cuda")
    check(lib().fv_rcm_permutation(n_cells, ptr(indptr), ptr(indices), ptr(seeds), ptr(perm),
                                   ptr(work), _stream()))
    return perm.cpu().numpy().astype(np.int64)


def mesh_rcm_permutation(mesh) -> np.ndarray:
    """:func:`rcm_permutation` of a :class:`aquaflux_gb300.mesh.MeshData`."""
    return rcm_permutation(mesh.owner, mesh.neighbour, mesh.n_cells)
