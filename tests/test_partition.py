"""Partitioned residual on the CPU: owned + ghost-layer partitions, the residual / JVP / VJP
evaluated partition by partition (the oracle as each partition's evaluator; for the SST channel
with the global wall distance) equal the serial oracle's, in one process and across two ``gloo``
ranks exchanging ghost rows point to point
(the reference's distributed = serial check, ``tests/unit/test_distributed.py:22-75``, there to
1e-10 / 1e-9, here to 1e-12)."""
from __future__ import annotations

import os

import numpy as np
import pytest
import torch

from aquaflux_gb300 import mesh as fm
from aquaflux_gb300.partition import (CUT_PATCH, DistributedResidual, PartitionedResidual,
                                      build_partitions, ghost_layers_needed, local_flow_bc,
                                      partition_cells)
from oracle import fv_oracle as fo

CAVITY_BC = {"top": ("moving", (1.0, 0.0)), "bottom": ("wall",), "left": ("wall",),
             "right": ("wall",)}
SPECS = {
    "compact": dict(gradient=None, advection=None),
    "corrected": dict(gradient={"sweeps": 4, "relaxation": 1.0}, advection=None),
    "limited": dict(gradient=None, advection={"k": 5.0}),
}


def _mesh(n=20, seed=0):
    m = fm.structured_grid_2d(n, n)
    m = m.with_nodes(fm.jitter_interior_nodes(m.nodes, (n, n), (1.0, 1.0), 0.15, seed))
    # a scrambled-then-blocked order is not needed: contiguous blocks of the natural order
    return m


class OracleLocal:
    """The oracle on a partition's local mesh (pin kept where the pinned cell is local)."""

    def __init__(self, part, spec, pin=0):
        hit = np.flatnonzero(part.cells == pin)
        case = fo.make_case(part.mesh, mu=0.01, rho=1.0, flow_bc=local_flow_bc(CAVITY_BC, part),
                            pressure_pin=int(hit[0]) if hit.size else None, **spec)
        self.orc = fo.Oracle(case)

    def residual(self, s):
        return self.orc.residual(torch.as_tensor(s, dtype=torch.float64)).detach()

    def jvp(self, s, v):
        return self.orc.jvp(s, v)

    def vjp(self, s, w):
        return self.orc.vjp(s, w).detach()


def _serial(m, spec):
    return fo.Oracle(fo.make_case(m, mu=0.01, rho=1.0, flow_bc=CAVITY_BC, pressure_pin=0, **spec))


def _layers(spec):
    sweeps = spec["gradient"]["sweeps"] if spec["gradient"] else 0
    return ghost_layers_needed(sweeps, spec["advection"] is not None)


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_partitions_cover_the_mesh_with_breadth_first_ghost_layers():
    m = _mesh(12)
    parts = build_partitions(m, partition_cells(m.n_cells, 3), 3)
    owned = np.concatenate([p.cells[p.owned] for p in parts])
    assert np.array_equal(np.sort(owned), np.arange(m.n_cells))
    ip, ix = fm.cell_adjacency_csr(m)
    for p in parts:
        layer_of = dict(zip(p.cells.tolist(), p.layer.tolist()))
        for c, k in layer_of.items():  # every ghost touches the previous layer
            if k > 0:
                nb = ix[ip[c]:ip[c + 1]]
                assert min(layer_of.get(int(x), 99) for x in nb) == k - 1
        assert p.mesh.n_cells == p.cells.size
        assert (CUT_PATCH in p.mesh.patches) == (p.layer.max() == 3 and p.cells.size < m.n_cells)


@pytest.mark.parametrize("name", list(SPECS))
def test_partitioned_evaluation_equals_serial(name):
    spec = SPECS[name]
    m = _mesh(20)
    serial = _serial(m, spec)
    pr = PartitionedResidual(m, 3, 3, _layers(spec), lambda p: OracleLocal(p, spec), device="cpu")
    rng = np.random.default_rng(1)
    s = rng.standard_normal(3 * m.n_cells) * 0.3
    v = rng.standard_normal(3 * m.n_cells)
    w = rng.standard_normal(3 * m.n_cells)
    assert _rel(pr.residual(s), serial.residual(torch.as_tensor(s)).detach()) <= 1e-12
    assert _rel(pr.jvp(s, v), serial.jvp(s, v)) <= 1e-12
    assert _rel(pr.vjp(s, w), serial.vjp(s, w).detach()) <= 1e-12


def test_too_few_ghost_layers_break_the_owned_rows():
    """The layer count is the reach: two layers leave owned rows next to the cut wrong."""
    spec = SPECS["compact"]
    m = _mesh(20)
    serial = _serial(m, spec)
    pr = PartitionedResidual(m, 3, 3, 2, lambda p: OracleLocal(p, spec), device="cpu")
    s = np.random.default_rng(1).standard_normal(3 * m.n_cells) * 0.3
    assert _rel(pr.residual(s), serial.residual(torch.as_tensor(s)).detach()) > 1e-10


def _gloo_problem(which):
    """(mesh, fields, ghost layers, make_local, serial oracle, state) of a two-rank test."""
    if which == "cavity":
        spec = SPECS["corrected"]
        m = _mesh(20)
        s = np.random.default_rng(1).standard_normal(3 * m.n_cells) * 0.3
        return m, 3, _layers(spec), (lambda p: OracleLocal(p, spec)), _serial(m, spec), s
    from aquaflux_gb300 import workloads

    wl = workloads.channel3d(4, 4, 24, renumber=False)
    serial = fo.Oracle(fo.make_case(wl.mesh, mu=wl.mu, rho=wl.rho, flow_bc=wl.flow_bc,
                                    sst=dict(wl.sst, nu=wl.mu / wl.rho)))
    gd = serial.wall_d.numpy()
    return (wl.mesh, 6, ghost_layers_needed(), (lambda p: _sst_oracle_local(wl, p, gd)), serial,
            wl.initial_state(seed=2, noise=0.05))


def _rank_main(rank, world, port, out_dir, which):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        m, nfld, layers, make_local, _, s = _gloo_problem(which)
        dr = DistributedResidual(m, nfld, layers, make_local, rank=rank, world=world)
        rng = np.random.default_rng(1)
        v = rng.standard_normal(s.size)
        w = rng.standard_normal(s.size)
        so, vo, wo = dr.owned_of(s), dr.owned_of(v), dr.owned_of(w)
        res = {"r": dr.residual(so), "jv": dr.jvp(so, vo), "g": dr.vjp(so, wo),
               "dot": torch.tensor(dr.dot(vo, wo), dtype=torch.float64), "cells": torch.as_tensor(
                   dr.part.cells[dr.part.owned])}
        torch.save(res, os.path.join(out_dir, f"rank{rank}.pt"))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("which", ["cavity", "sst"])
def test_two_gloo_ranks_equal_serial(tmp_path, which):
    """Two gloo ranks: the corrected-gradient cavity, and the SST channel with the global wall
    distance."""
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path), which), nprocs=2,
                       start_method="spawn")
    m, nfld, _, _, serial, s = _gloo_problem(which)
    rng = np.random.default_rng(1)
    v = rng.standard_normal(s.size)
    w = rng.standard_normal(s.size)
    want = {"r": serial.residual(torch.as_tensor(s)).detach().numpy(),
            "jv": serial.jvp(s, v).numpy(), "g": serial.vjp(s, w).detach().numpy()}
    got = {k: np.zeros(s.size) for k in want}
    dots = []
    for rank in range(2):
        res = torch.load(os.path.join(tmp_path, f"rank{rank}.pt"))
        cells = res["cells"].numpy()
        for k in want:
            got[k].reshape(nfld, -1)[:, cells] = res[k].numpy().reshape(nfld, -1)
        dots.append(float(res["dot"]))
    for k in want:
        assert _rel(got[k], want[k]) <= 1e-12, k
    assert dots[0] == dots[1]
    assert abs(dots[0] - float(np.dot(v, w))) <= 1e-12 * abs(float(np.dot(np.abs(v), np.abs(w))))


def test_halo_plans_pair_up():
    """What rank p receives from q is what q sends to p: the same global cells, in the same order."""
    from aquaflux_gb300.partition import halo_plans

    m = _mesh(16)
    owner = partition_cells(m.n_cells, 4)
    parts = build_partitions(m, owner, 3)
    plans = halo_plans(parts, owner)
    for p in parts:
        for q, local in plans[p.rank].recv.items():
            want = p.cells[local]
            qp = parts[q]
            sent = qp.cells[qp.owned][plans[q].send[p.rank]]
            assert np.array_equal(want, sent)
            assert np.all(owner[want] == q)
    # every ghost is received from exactly its owner
    for p in parts:
        got = np.concatenate([p.cells[v] for v in plans[p.rank].recv.values()]) \
            if plans[p.rank].recv else np.zeros(0, dtype=np.int64)
        assert np.array_equal(np.sort(got), np.sort(p.cells[p.ghosts]))


def _sst_oracle_local(wl, part, global_d):
    """The oracle on a partition of an SST workload, with the global wall distance on its cells
    and that distance's Green-Gauss gradient formed on the local mesh (walls Dirichlet 0, every
    other boundary, the cut included, zero gradient), as ``fv_case_set_wall_distance`` does."""
    from aquaflux_gb300.partition import local_sst

    sst = dict(local_sst(wl.sst, part), nu=wl.mu / wl.rho)
    case = fo.make_case(part.mesh, mu=wl.mu, rho=wl.rho, flow_bc=local_flow_bc(wl.flow_bc, part),
                        sst=sst)
    orc = fo.Oracle(case)
    geo = fo.geometry(orc.topo, orc.nodes)
    d = torch.as_tensor(np.asarray(global_d)[part.cells], dtype=torch.float64)
    is_wall = np.zeros(orc.topo.n_faces, dtype=bool)
    is_wall[case["sst"]["wall_faces"]] = True
    bvals = torch.where(torch.as_tensor(is_wall), torch.zeros(orc.topo.n_faces, dtype=torch.float64),
                        d[orc.topo.owner])
    orc.wall_d = d
    orc.wall_dgrad = fo.gg_gradient(fo.Metrics(orc.topo, geo), d, bvals, case.get("gradient"))

    class Local:
        def residual(self, s):
            return orc.residual(torch.as_tensor(s, dtype=torch.float64)).detach()

        def jvp(self, s, v):
            return orc.jvp(s, v)

        def vjp(self, s, w):
            return orc.vjp(s, w).detach()

    return Local()


def test_partitioned_sst_channel_equals_serial():
    """The coupled SST channel split into three slabs along its length, each evaluated on its own
    mesh with the global wall distance: residual, JVP and VJP equal the serial oracle's."""
    from aquaflux_gb300 import workloads

    wl = workloads.channel3d(4, 4, 24, renumber=False)  # slabs along the channel
    m = wl.mesh
    sst = dict(wl.sst, nu=wl.mu / wl.rho)
    serial = fo.Oracle(fo.make_case(m, mu=wl.mu, rho=wl.rho, flow_bc=wl.flow_bc, sst=sst))
    gd = serial.wall_d.numpy()
    n_parts = 3
    parts = build_partitions(m, partition_cells(m.n_cells, n_parts), ghost_layers_needed())
    assert all(any(w in p.mesh.patches for w in wl.sst["walls"]) for p in parts)
    # proper subsets: a partition's own nearest wall is not always the global one (the local
    # distance alone leaves ~5e-6 relative errors in the owned rows)
    assert all(p.cells.size < m.n_cells for p in parts)
    pr = PartitionedResidual(m, 6, n_parts, ghost_layers_needed(),
                             lambda p: _sst_oracle_local(wl, p, gd), device="cpu")
    rng = np.random.default_rng(5)
    s = wl.initial_state(seed=2, noise=0.05)
    v = rng.standard_normal(s.size)
    w = rng.standard_normal(s.size)
    assert _rel(pr.residual(s), serial.residual(torch.as_tensor(s)).detach()) <= 1e-12
    assert _rel(pr.jvp(s, v), serial.jvp(s, v)) <= 1e-12
    assert _rel(pr.vjp(s, w), serial.vjp(s, w).detach()) <= 1e-12
