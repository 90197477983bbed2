"""Pseudo-transient continuation: the shifted march converges where Newton from a cold start does
not, to the same root a viscosity continuation of Newton reaches."""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_shift_basis_is_the_momentum_diagonal():
    from aquaflux_gb300 import workloads
    from aquaflux_gb300.solve import BlockJacobian, shift_basis

    wl = workloads.channel3d(6, nu=1e-2)
    case = wl.device_case()
    jac = BlockJacobian(case)
    s = torch.tensor(wl.initial_state(), device="cuda")
    jac.materialize(s)
    d = shift_basis(jac).view(6, -1)
    A = jac.to_scipy().tocsr()
    n = jac.n
    diag = np.abs(A.diagonal()).reshape(n, 6).T
    assert torch.equal(d[:3].cpu(), torch.tensor(diag[:3]))
    assert float(d[3].abs().max()) == 0.0
    assert torch.equal(d[4:].cpu(), torch.tensor(diag[4:]))


@pytest.mark.parametrize("kind", ["ilu", "amg"])
def test_pseudo_transient_converges_high_reynolds_cavity(kind):
    from aquaflux_gb300 import workloads
    from aquaflux_gb300.solve import newton_solve, pseudo_transient_solve

    wl = workloads.cavity(32, mu=1e-3)  # Re = 1000 from the zero state
    case = wl.device_case()
    ptc = pseudo_transient_solve(case, np.zeros(case.n_unknowns), kind=kind, precision=32,
                                 max_steps=200)
    assert ptc.converged
    assert ptc.betas[-1] < ptc.betas[0]
    # the root by Newton, continued in viscosity from Re = 100
    s = np.zeros(case.n_unknowns)
    for mu in (1e-2, 3e-3, 1e-3):
        case.set_params(mu=mu)
        res = newton_solve(case, s, precision=64, max_steps=60)
        assert res.converged
        s = res.state
    a, b = ptc.state.cpu().numpy(), s.cpu().numpy()
    assert np.abs(a - b).max() <= 1e-7 * np.abs(b).max()
