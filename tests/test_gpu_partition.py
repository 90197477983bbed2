"""The partitioned residual on the GPU: every partition's local mesh (owned cells + ghost layers)
evaluated by the library's kernels, the owned rows gathered -- equal to the serial evaluation
(residual, JVP, VJP), for the SST channel with the global wall distance, corrected Green-Gauss and
limited upwind."""
from __future__ import annotations

import dataclasses

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = a.detach().cpu().numpy(), b.detach().cpu().numpy()
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("name,n_parts", [("sst_channel", 4), ("corrected_channel", 3),
                                          ("limited_cavity", 3)])
def test_partitioned_gpu_evaluation_equals_serial(name, n_parts):
    from aquaflux_gb300 import workloads
    from aquaflux_gb300.partition import (PartitionedResidual, flow_case_factory,
                                          ghost_layers_needed)

    if name == "sst_channel":
        wl = workloads.channel3d(10)
    elif name == "corrected_channel":
        wl = dataclasses.replace(workloads.channel3d(8, nu=1e-2),
                                 gradient={"sweeps": 3, "relaxation": 0.9})
    else:
        wl = dataclasses.replace(workloads.cavity(24), advection={"k": 5.0})
    serial = wl.device_case()
    wd = serial.wall_distance()[0].cpu().numpy() if wl.sst is not None else None
    sweeps = wl.gradient["sweeps"] if wl.gradient else 0
    layers = ghost_layers_needed(sweeps, wl.advection is not None)
    nfld = serial.n_unknowns // serial.n_cells
    pr = PartitionedResidual(wl.mesh, nfld, n_parts, layers, flow_case_factory(wl, wd))
    rng = np.random.default_rng(3)
    s = torch.tensor(wl.initial_state(seed=2, noise=0.05), device="cuda")
    v = torch.tensor(rng.standard_normal(s.numel()), device="cuda")
    w = torch.tensor(rng.standard_normal(s.numel()), device="cuda")
    assert _rel(pr.residual(s), serial.residual(s)) <= 1e-12
    assert _rel(pr.jvp(s, v), serial.jvp(s, v)) <= 1e-12
    assert _rel(pr.vjp(s, w), serial.vjp(s, w)) <= 1e-12


def test_wall_less_turbulent_partition_needs_its_distance():
    from aquaflux_gb300 import fv, workloads
    from aquaflux_gb300._lib import FvError
    from aquaflux_gb300.partition import build_partitions, local_flow_bc, local_sst, \
        partition_cells

    wl = workloads.channel3d(16, renumber=False)
    parts = build_partitions(wl.mesh, partition_cells(wl.mesh.n_cells, 8), 3)
    # natural order: blocks are x-slabs; the inner ones touch the walls, so strip the walls from
    # the SST description to make a case without SST wall faces
    p = parts[3]
    sst = local_sst(wl.sst, p)
    sst["walls"] = []
    case = fv.FlowCase(fv.DeviceMesh(p.mesh), mu=wl.mu, rho=wl.rho,
                       flow_bc=local_flow_bc(wl.flow_bc, p), sst=sst)
    s = np.ones(case.n_unknowns)
    with pytest.raises(FvError):
        case.residual(s)
    case.set_wall_distance(np.full(case.n_cells, 0.1))
    assert torch.isfinite(case.residual(s)).all()
