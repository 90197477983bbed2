"""Flow on imported polyMeshes: a 2D case written one cell thick (``empty`` caps) and a 3D case go
through the OpenFOAM import and give the residual, VJP and Newton solution of the same case on the
native mesh, and the oracle's residual on the imported mesh."""
from __future__ import annotations

import dataclasses

import numpy as np
import pytest
import torch

from aquaflux_gb300 import openfoam as of
from aquaflux_gb300 import workloads
from oracle import fv_oracle as fo
from tests.cases import workload_oracle_case

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = b.detach().cpu().numpy() if torch.is_tensor(b) else np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _import(wl, tmp_path, types, caps=None):
    mesh = wl.mesh
    if mesh.dim == 2:
        mesh = of.extrude_2d(mesh, 0.05, caps=caps)
    of.write_polymesh(mesh, tmp_path / "constant" / "polyMesh", types)
    back = of.read_openfoam(tmp_path)
    assert back.dim == wl.mesh.dim and back.n_cells == wl.mesh.n_cells
    return dataclasses.replace(wl, mesh=back)


@pytest.mark.parametrize("caps", [("frontAndBack",), ("front", "back")])
def test_imported_backward_step_matches_native(tmp_path, caps):
    wl = workloads.backward_step(n_step=8, n_channel=12, n_upstream=10, n_downstream=40)
    types = {**{c: "empty" for c in caps}, "step": "wall", "top": "wall", "bottom": "wall"}
    wi = _import(wl, tmp_path, types, caps)
    fc, fi = wl.device_case(), wi.device_case()
    s = wl.initial_state(noise=0.05)
    ri = fi.residual(s)
    assert _rel(ri, fc.residual(s)) <= 1e-12
    assert _rel(ri, fo.Oracle(workload_oracle_case(wi)).residual(torch.as_tensor(s))) <= 1e-12
    w = np.random.default_rng(3).standard_normal(s.size)
    assert _rel(fi.vjp(s, w), fc.vjp(s, w)) <= 1e-11


def test_imported_3d_channel_matches_native(tmp_path):
    wl = workloads.channel3d(10, 6, 6)
    wi = _import(wl, tmp_path, {"bottom": "wall", "top": "wall", "back": "wall", "front": "wall"})
    fc, fi = wl.device_case(), wi.device_case()
    s = wl.initial_state(noise=0.05)
    assert _rel(fi.residual(s), fc.residual(s)) <= 1e-12
    v = np.random.default_rng(4).standard_normal(s.size)
    assert _rel(fi.jvp(s, v), fc.jvp(s, v)) <= 1e-11


def test_newton_on_imported_cavity_matches_native(tmp_path):
    from aquaflux_gb300.solve import newton_solve

    wl = workloads.cavity(24, mu=0.01)
    wi = _import(wl, tmp_path, {"front": "empty", "back": "empty"}, ("front", "back"))
    s0 = wl.initial_state()
    a = newton_solve(wl.device_case(), s0, precision=64)
    b = newton_solve(wi.device_case(), s0, precision=64)
    assert a.converged and b.converged
    assert _rel(b.state, a.state) <= 1e-8
