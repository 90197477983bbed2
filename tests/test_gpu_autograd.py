"""The torch.autograd.Function binding against the oracle's autograd (state, viscosity, inlet
scale, node coordinates)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import fv_oracle as fo
from tests.cases import device_case

pytestmark = pytest.mark.gpu


def _moved(nodes, seed, amount):
    """The nodes moved by a small seeded perturbation (relative to the mesh extent)."""
    ext = nodes.max(0) - nodes.min(0)
    return nodes + np.random.default_rng(seed).uniform(-1, 1, nodes.shape) * amount * ext


@pytest.mark.parametrize("name,move", [("cavj", 0.0), ("lam3", 0.0), ("sst2", 0.0),
                                       ("sst3", 0.0), ("sst2", 1e-3), ("sst3", 1e-3)])
def test_autograd_function_matches_oracle(name, move):
    from aquaflux_gb300.autograd import residual

    fc, case, d, p = device_case(name)
    s0 = d[p + "states"][0]
    w = np.random.default_rng(0).standard_normal(s0.size)
    state = torch.tensor(s0, device="cuda", requires_grad=True)
    mu = torch.tensor(case["mu"], dtype=torch.float64, requires_grad=True)
    sc = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    x = _moved(d[p + "nodes"], 7, move) if move else d[p + "nodes"]
    nodes = torch.tensor(x, device="cuda", requires_grad=True)
    r = residual(fc, state, mu, sc, nodes)
    (r * torch.tensor(w, device="cuda")).sum().backward()

    orc = fo.Oracle(case)
    so = torch.tensor(s0, requires_grad=True)
    muo = torch.tensor(case["mu"], dtype=torch.float64, requires_grad=True)
    sco = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    no = torch.tensor(x, requires_grad=True)
    ro = orc.residual(so, mu=muo, inlet_scale=sco, nodes=no)
    (ro * torch.tensor(w)).sum().backward()

    def rel(a, b):
        a, b = a.detach().cpu().numpy(), b.detach().cpu().numpy()
        return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))

    assert rel(r, ro) <= 1e-12
    assert rel(state.grad, so.grad) <= 1e-11
    assert abs(float(mu.grad) - float(muo.grad)) <= 1e-10 * max(1.0, abs(float(muo.grad)))
    assert abs(float(sc.grad) - float(sco.grad)) <= 1e-10 * max(1.0, abs(float(sco.grad)))
    assert rel(nodes.grad, no.grad) <= 1e-10


@pytest.mark.parametrize("name", ["sst2", "sst3"])
def test_autograd_node_gradient_matches_central_differences_sst(name):
    """The forward under moved nodes and the backward describe the same function: w . R through
    the autograd binding at x +- h v (geometry and SST wall distance recomputed on the GPU)
    against the binding's own node gradient."""
    from aquaflux_gb300.autograd import residual

    fc, case, d, p = device_case(name)
    s0 = torch.tensor(d[p + "states"][0], device="cuda")
    rng = np.random.default_rng(11)
    w = torch.tensor(rng.standard_normal(s0.numel()), device="cuda")
    x0 = d[p + "nodes"]
    v = torch.tensor(rng.standard_normal(x0.shape) * 1e-2 * (x0.max(0) - x0.min(0)),
                     device="cuda")
    nodes = torch.tensor(x0, device="cuda", requires_grad=True)
    (residual(fc, s0, nodes=nodes) * w).sum().backward()
    exact = float((nodes.grad * v).sum())
    h = 1e-6

    def wr(sign):
        xn = torch.tensor(x0, device="cuda") + sign * h * v
        return float((residual(fc, s0, nodes=xn) * w).sum())

    fd = (wr(1.0) - wr(-1.0)) / (2 * h)
    residual(fc, s0, nodes=torch.tensor(x0, device="cuda"))
    assert abs(fd - exact) <= 1e-6 * max(abs(exact), 1.0), (fd, exact)
