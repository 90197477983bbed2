"""Face-flux functionals (outlet mass flux, wall shear force) and their total gradients with
respect to viscosity, inlet velocity and every node coordinate by the implicit function theorem,
against finite differences of re-converged solves."""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

WALLS = ["bottom", "top", "back", "front"]


def _shear_spec(dim):
    return {w: {0: 1.0} for w in WALLS}


def _outlet_spec(dim):
    return {"right": {dim: 1.0}}


def test_functional_partials_match_finite_differences():
    """dJ/dstate and dJ/dnodes at fixed state against central differences (laminar duct)."""
    from aquaflux_gb300._lib import check, lib, ptr
    from tests.cases import device_case

    fc, case, d, p = device_case("lam3")
    s = d[p + "states"][0]
    rng = np.random.default_rng(1)
    for spec, visc in ((_shear_spec(3), True), (_outlet_spec(3), False)):
        w = fc.functional_weights({k: v for k, v in spec.items() if k in fc.dmesh.mesh.patches})
        out = fc.face_functional(s, w, viscous_only=visc)
        v = rng.standard_normal(s.size)
        h = 1e-6
        jp = fc.face_functional(s + h * v, w, viscous_only=visc, nodes=False)["value"]
        jm = fc.face_functional(s - h * v, w, viscous_only=visc, nodes=False)["value"]
        exact = float(torch.dot(out["dstate"], torch.tensor(v, device="cuda")))
        assert abs((jp - jm) / (2 * h) - exact) <= 1e-6 * max(abs(exact), 1e-3)
        nodes = d[p + "nodes"]
        dx = rng.standard_normal(nodes.shape) * 1e-2

        def jn(x):
            xd = torch.tensor(x, device="cuda")
            check(lib().fv_mesh_set_nodes(fc.dmesh.handle, ptr(xd),
                                          torch.cuda.current_stream().cuda_stream))
            return fc.face_functional(s, w, viscous_only=visc, nodes=False)["value"]

        fd = (jn(nodes + h * dx) - jn(nodes - h * dx)) / (2 * h)
        jn(nodes)
        exact = float((out["dnodes"].cpu().numpy() * dx).sum())
        assert abs(fd - exact) <= 1e-6 * max(abs(exact), 1e-3)


def _solve(wl, mesh=None, mu=None, inlet=None):
    from aquaflux_gb300 import fv
    from aquaflux_gb300.solve import newton_solve

    dm = fv.DeviceMesh(wl.mesh if mesh is None else mesh)
    case = fv.FlowCase(dm, mu=wl.mu if mu is None else mu, rho=wl.rho, flow_bc=wl.flow_bc,
                       pressure_pin=wl.pressure_pin, sst=wl.sst)
    if inlet is not None:
        case.set_params(inlet_scale=inlet)
    res = newton_solve(case, wl.initial_state(), precision=64, rtol=1e-13, atol=1e-14,
                       max_steps=60)
    assert res.converged
    return case, res.state


@pytest.mark.parametrize("kind", ["shear", "outlet"])
def test_ift_gradients_match_resolved_finite_differences(kind):
    """The channel's adjoint objectives (config 3's form at 6^3): dJ/dmu, dJ/d inlet scale and
    dJ/dnodes . v against central differences of J at re-converged states."""
    from aquaflux_gb300 import workloads
    from aquaflux_gb300.solve import functional_gradient

    wl = workloads.channel3d(6, nu=2e-2)
    case, s = _solve(wl)
    spec = _shear_spec(3) if kind == "shear" else _outlet_spec(3)
    visc = kind == "shear"
    w = case.functional_weights(spec)
    g = functional_gradient(case, s, w, viscous_only=visc, rtol=1e-13)

    def J(case_, state):
        return case_.face_functional(state, case_.functional_weights(spec), viscous_only=visc,
                                     params=False, nodes=False)["value"]

    h = 1e-5
    fd_mu = (J(*_solve(wl, mu=wl.mu * (1 + h))) - J(*_solve(wl, mu=wl.mu * (1 - h)))) / (2 * h * wl.mu)
    fd_in = (J(*_solve(wl, inlet=1 + h)) - J(*_solve(wl, inlet=1 - h))) / (2 * h)
    scale = max(abs(fd_mu), abs(fd_in), abs(g.value), 1e-8)
    assert abs(float(g.dparams[0]) - fd_mu) <= 1e-5 * scale
    assert abs(float(g.dparams[1]) - fd_in) <= 1e-5 * scale
    rng = np.random.default_rng(3)
    dx = rng.standard_normal(wl.mesh.nodes.shape) * 1e-2
    hx = 1e-4
    fd_x = (J(*_solve(wl, mesh=wl.mesh.with_nodes(wl.mesh.nodes + hx * dx))) -
            J(*_solve(wl, mesh=wl.mesh.with_nodes(wl.mesh.nodes - hx * dx)))) / (2 * hx)
    exact = float((g.dnodes.cpu().numpy() * dx).sum())
    assert abs(fd_x - exact) <= 1e-5 * max(abs(exact), abs(fd_x), 1e-8)
