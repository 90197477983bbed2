"""Batched instances in one disjoint-union mesh (host side)."""
import numpy as np

from aquaflux_gb300 import mesh as fm
from aquaflux_gb300 import workloads


def test_disjoint_union_keeps_every_instance():
    a = fm.structured_grid_2d(3, 2)
    b = fm.structured_grid_2d(4, 5, 2.0, 1.0)
    u, off = fm.disjoint_union([a, b])
    assert list(off) == [0, 6, 26]
    assert u.n_faces == a.n_faces + b.n_faces and u.n_nodes == a.n_nodes + b.n_nodes
    assert np.array_equal(u.owner[a.n_faces:], b.owner + 6)
    nb = u.neighbour[a.n_faces:]
    assert np.array_equal(nb[nb >= 0], b.neighbour[b.neighbour >= 0] + 6)
    assert np.array_equal(u.patches["1:left"], b.patches["left"] + a.n_faces)
    assert np.array_equal(u.nodes[a.n_nodes:], b.nodes)


def test_batched_channels_sizes_and_parameters():
    bw = workloads.batched_channels(64, seed=0)
    assert bw.n_instances == 64
    assert bw.sizes.min() >= 32 and bw.sizes.max() <= 256
    assert 1e-3 <= bw.mu.min() and bw.mu.max() <= 1e-1
    assert 0.5 <= bw.velocity.min() and bw.velocity.max() <= 2.0
    assert bw.workload.mesh.n_cells == int((bw.sizes ** 2).sum())
    assert 3e5 < bw.workload.mesh.n_cells < 3e6
    again = workloads.batched_channels(64, seed=0)
    assert np.array_equal(again.mu, bw.mu) and np.array_equal(again.sizes, bw.sizes)
