"""Reverse Cuthill-McKee on the GPU against scipy's ``reverse_cuthill_mckee`` (the reference's
``ReverseCuthillMcKee``, ``aquaflux/mesh/reorder.py:147-159``): the cell graph and the
permutation bit for bit, on randomly relabelled 2D / 3D meshes, a disconnected mesh (one sweep
per component) and the randomly permuted 128^3 benchmark channel."""
from __future__ import annotations

import numpy as np
import pytest

from aquaflux_gb300 import mesh as fm
from aquaflux_gb300 import workloads

pytestmark = pytest.mark.gpu


def _scrambled(m, seed):
    return fm.permute_cells(m, fm.random_permutation(m.n_cells, seed))


def test_cell_graph_matches_the_host_adjacency():
    from aquaflux_gb300.reorder import cell_graph

    m = _scrambled(workloads.channel3d(9, 7, 5, renumber=False).mesh, 4)
    ip, ix = fm.cell_adjacency_csr(m)
    gp, gi = cell_graph(m.owner, m.neighbour, m.n_cells)
    assert np.array_equal(gp.cpu().numpy(), ip) and np.array_equal(gi.cpu().numpy(), ix)


@pytest.mark.parametrize("name", ["channel3d_12", "square_40", "graded_step", "batched"])
def test_rcm_permutation_equals_scipy(name):
    from aquaflux_gb300.reorder import mesh_rcm_permutation

    if name == "channel3d_12":
        m = _scrambled(workloads.channel3d(12, renumber=False).mesh, 1)
    elif name == "square_40":
        m = _scrambled(fm.structured_grid_2d(40, 40), 2)
    elif name == "graded_step":
        m = _scrambled(fm.backward_step_2d(n_step=6, n_channel=10, n_upstream=12,
                                           n_downstream=40, seed=0), 3)
    else:  # disconnected: uneven instances side by side
        m = _scrambled(workloads.batched_channels(6, n_min=4, n_max=12, seed=5).workload.mesh, 4)
    assert np.array_equal(mesh_rcm_permutation(m), workloads.rcm_permutation(m))


def test_rcm_permutation_equals_scipy_on_the_128_channel():
    """The benchmark mesh: 2,097,152 cells, randomly relabelled, then renumbered on the GPU."""
    from aquaflux_gb300.reorder import mesh_rcm_permutation

    m = _scrambled(workloads.channel3d(128, renumber=False).mesh, 0)
    assert np.array_equal(mesh_rcm_permutation(m), workloads.rcm_permutation(m))


def test_cell_graph_refuses_bad_pairs():
    from aquaflux_gb300._lib import FvError
    from aquaflux_gb300.reorder import cell_graph

    with pytest.raises(FvError):
        cell_graph(np.array([0, 1]), np.array([1, 5]), 3)
    with pytest.raises(FvError):
        cell_graph(np.array([0, 2]), np.array([1, 2]), 3)
