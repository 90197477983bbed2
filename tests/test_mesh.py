"""The package's structured generators and node recipes against the reference's own meshes."""
from __future__ import annotations

import numpy as np
import pytest

from aquaflux_gb300 import mesh as fm
from tests.cases import golden


def _check(m: fm.MeshData, d: dict, p: str):
    np.testing.assert_array_equal(m.owner, d[p + "owner"])
    np.testing.assert_array_equal(m.neighbour, d[p + "neighbour"])
    np.testing.assert_array_equal(m.fn_offsets, d[p + "fn_offsets"])
    np.testing.assert_array_equal(m.fn_indices, d[p + "fn_indices"])
    np.testing.assert_array_equal(m.nodes, d[p + "nodes"])  # bit-identical coordinates
    names = {k[len(p) + 6:] for k in d if k.startswith(p + "patch_")}
    for name in names - {"interior", "boundary"}:
        np.testing.assert_array_equal(m.patches[name], d[p + "patch_" + name])


def test_jittered_2d():
    m = fm.structured_grid_2d(5, 4, lx=2.0, ly=1.0)
    m = m.with_nodes(fm.jitter_interior_nodes(m.nodes, (5, 4), (2.0, 1.0), 0.15, 3))
    _check(m, golden("meshes"), "m2d_")


def test_bump_3d():
    m = fm.structured_grid_3d(4, 3, 3, lx=2.0, ly=1.0, lz=1.0)
    m = m.with_nodes(fm.bump_channel_nodes_3d((4, 3, 3), (2.0, 1.0, 1.0), 0.1, 0.1, 5))
    _check(m, golden("meshes"), "m3d_")


def test_graded_2d():
    d = golden("meshes")
    yn = fm.graded_nodes(6, 1.0, 1.3)
    np.testing.assert_array_equal(yn, d["mgr_y_nodes"])
    _check(fm.structured_grid_2d(7, 6, lx=3.0, ly=1.0, y_nodes=yn), d, "mgr_")


@pytest.mark.parametrize("case", ["cav8", "cavj", "lam3"])
def test_residual_case_meshes(case):
    d = golden("laminar")
    if case == "cav8":
        m = fm.structured_grid_2d(8, 8)
    elif case == "cavj":
        m = fm.structured_grid_2d(10, 10)
        m = m.with_nodes(fm.jitter_interior_nodes(m.nodes, (10, 10), (1.0, 1.0), 0.15, 0))
    else:
        m = fm.structured_grid_3d(4, 3, 3, 2.0, 1.0, 1.0)
        m = m.with_nodes(fm.bump_channel_nodes_3d((4, 3, 3), (2.0, 1.0, 1.0), 0.1, 0.1, 7))
    _check(m, d, case + "_")


def test_sst_meshes():
    d = golden("sst")
    yn = fm.graded_nodes(8, 1.0, 1.2)
    m = fm.structured_grid_2d(12, 8, lx=4.0, ly=1.0, y_nodes=yn)
    m = m.with_nodes(fm.jitter_interior_nodes(m.nodes, (12, 8), (4.0, 1.0), 0.1, 4))
    _check(m, d, "sst2_")
    m = fm.structured_grid_3d(5, 4, 3, 2.0, 1.0, 1.0)
    m = m.with_nodes(fm.bump_channel_nodes_3d((5, 4, 3), (2.0, 1.0, 1.0), 0.1, 0.1, 9))
    _check(m, d, "sst3_")


def test_permute_round_trip():
    m = fm.structured_grid_3d(3, 3, 2)
    perm = fm.random_permutation(m.n_cells, seed=4)
    p = fm.permute_cells(m, perm)
    back = fm.permute_cells(p, np.argsort(perm))
    np.testing.assert_array_equal(back.owner, m.owner)
    np.testing.assert_array_equal(back.neighbour, m.neighbour)


def test_validate_rejects_bad_topology():
    m = fm.structured_grid_2d(3, 3)
    bad = fm.MeshData(m.nodes, m.fn_offsets, m.fn_indices, m.owner.copy(), m.neighbour.copy(),
                      m.n_cells, m.patches)
    bad.owner[0] = m.n_cells
    with pytest.raises(ValueError):
        bad.validate()


def test_backward_step_mesh():
    """The two-block backward-facing-step generator: closed cells of positive volume filling the
    30h x 1.5h domain less the step, every boundary face in exactly one patch, seeded jitter."""
    import torch

    from aquaflux_gb300.mesh import backward_step_2d
    from oracle import fv_oracle as fo

    m = backward_step_2d(n_step=6, n_channel=8, n_upstream=6, n_downstream=20)
    assert m.n_cells == 8 * 26 + 6 * 20
    topo = fo.Topology(m.owner, m.neighbour, m.n_cells, m.fn_offsets, m.fn_indices)
    geo = fo.geometry(topo, torch.as_tensor(m.nodes))
    vol = geo["volume"].numpy()
    assert vol.min() > 0 and abs(vol.sum() - (30.0 * 1.5 - 5.0 * 0.5)) <= 1e-12
    bnd = np.flatnonzero(m.neighbour < 0)
    allp = np.concatenate([m.patches[k] for k in ("inlet", "outlet", "top", "bottom", "step")])
    assert np.array_equal(np.sort(allp), bnd)
    assert len(m.patches["step"]) == 6 + 6 and len(m.patches["inlet"]) == 8
    # closed cells: the area vectors of each cell's faces sum to zero
    s = (geo["normal"] * geo["area"][:, None]).numpy()
    tot = np.zeros((m.n_cells, 2))
    np.add.at(tot, m.owner, s)
    inner = m.neighbour >= 0
    np.add.at(tot, m.neighbour[inner], -s[inner])
    assert np.abs(tot).max() <= 1e-13
    again = backward_step_2d(n_step=6, n_channel=8, n_upstream=6, n_downstream=20)
    assert np.array_equal(again.nodes, m.nodes)
    other = backward_step_2d(n_step=6, n_channel=8, n_upstream=6, n_downstream=20, seed=1)
    assert not np.array_equal(other.nodes, m.nodes)
    full = backward_step_2d()
    assert 190_000 <= full.n_cells <= 210_000
