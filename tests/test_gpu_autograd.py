"""The torch.autograd.Function binding against the oracle's autograd (state, viscosity, inlet
scale, node coordinates)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import fv_oracle as fo
from tests.cases import device_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["cavj", "lam3"])
def test_autograd_function_matches_oracle(name):
    from aquaflux_gb300.autograd import residual

    fc, case, d, p = device_case(name)
    s0 = d[p + "states"][0]
    w = np.random.default_rng(0).standard_normal(s0.size)
    state = torch.tensor(s0, device="cuda", requires_grad=True)
    mu = torch.tensor(case["mu"], dtype=torch.float64, requires_grad=True)
    sc = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    nodes = torch.tensor(d[p + "nodes"], device="cuda", requires_grad=True)
    r = residual(fc, state, mu, sc, nodes)
    (r * torch.tensor(w, device="cuda")).sum().backward()

    orc = fo.Oracle(case)
    so = torch.tensor(s0, requires_grad=True)
    muo = torch.tensor(case["mu"], dtype=torch.float64, requires_grad=True)
    sco = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    no = torch.tensor(d[p + "nodes"], requires_grad=True)
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
