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


def test_fixation_rows_take_no_shift_and_the_row_scaled_measure():
    """The near-wall omega rows (FixedValueCells) are algebraic: no pseudo-time shift there
    (coupled.py:1098-1110); the row-scaled measure passes a log-ratio row through with its unit
    derivative and a log-solved field with field scale 1 (coupled_scaled_norm, coupled.py:1073)."""
    import dataclasses

    from aquaflux_gb300 import workloads
    from aquaflux_gb300.solve import BlockJacobian, RowScaledMeasure, shift_basis

    wl = dataclasses.replace(workloads.channel3d(6, nu=1e-2), omega_transform="log")
    case = wl.device_case()
    jac = BlockJacobian(case)
    s = torch.tensor(case.to_solved(wl.initial_state(noise=0.02)), device="cuda")
    jac.materialize(s)
    n = jac.n
    fixed = torch.as_tensor(5 * n + case.wall_cells, device="cuda")
    d = shift_basis(jac, fixed_rows=fixed)
    assert float(d[fixed].abs().max()) == 0.0
    free = torch.ones(6 * n, dtype=torch.bool, device="cuda")
    free[fixed] = False
    free[3 * n:4 * n] = False  # continuity
    assert float(d[free].min()) > 0.0
    meas = RowScaledMeasure(case, jac, s)
    assert torch.allclose(meas.row[fixed], torch.ones_like(meas.row[fixed]), rtol=1e-12)
    assert float(meas.field[5]) == 1.0  # log omega: a change of log omega is already relative
    r = case.residual(s)
    blocks = meas.per_block(r)
    assert abs(float(torch.linalg.vector_norm(blocks)) - meas(r)) <= 1e-12 * meas(r)
    manual = (r.abs() / meas.row).view(6, n).mean(dim=1) / meas.field
    assert torch.allclose(blocks, manual)


def test_row_scaled_march_with_backtracking_reaches_the_newton_root():
    """The SST channel from a cold start, steered by the row-scaled measure with k kept positive
    and backtracking before escalation, lands on the root plain Newton finds."""
    import dataclasses

    from aquaflux_gb300 import workloads
    from aquaflux_gb300.solve import newton_solve, pseudo_transient_solve

    wl = dataclasses.replace(workloads.channel3d(8, nu=2e-3), omega_transform="log")
    case = wl.device_case()
    s0 = case.to_solved(wl.initial_state())
    ptc = pseudo_transient_solve(case, s0, kind="amg", precision=64, max_steps=120,
                                 measure="row_scaled", k_positive=True, backtrack=4)
    assert ptc.converged
    ref = newton_solve(case, s0, precision=64, max_steps=60)
    assert ref.converged
    a, b = ptc.state.cpu().numpy(), ref.state.cpu().numpy()
    assert np.abs(a - b).max() <= 1e-7 * np.abs(b).max()


@pytest.mark.parametrize("trigger", ["cycles", "drift"])
def test_triggered_refresh_reaches_the_same_root(trigger):
    """A march whose Jacobian is re-materialised only when a staleness trigger fires (the steps
    between re-shift the frozen Jacobian) converges to the root of the every-step march; the
    cycle-growth trigger on the Re = 1000 cavity, the eddy-viscosity drift trigger on an SST
    channel."""
    from aquaflux_gb300 import workloads
    from aquaflux_gb300.refresh import (CoefficientDriftTrigger, CycleGrowthTrigger,
                                        eddy_viscosity_drift)
    from aquaflux_gb300.solve import pseudo_transient_solve

    if trigger == "cycles":
        wl = workloads.cavity(32, mu=1e-3)
        case = wl.device_case()
        s0 = np.zeros(case.n_unknowns)
        kw = dict(refresh_trigger=CycleGrowthTrigger(warmup=2, patience=1,
                                                     max_residual_ratio=1.0))
    else:
        wl = workloads.channel3d(6, nu=1e-2)
        case = wl.device_case()
        s0 = wl.initial_state()
        kw = dict(refresh_trigger=CoefficientDriftTrigger(threshold=0.05, warmup=1),
                  drift_measure=eddy_viscosity_drift(case))
    every = pseudo_transient_solve(case, s0, kind="ilu", precision=64, max_steps=300)
    lazy = pseudo_transient_solve(case, s0, kind="ilu", precision=64, max_steps=300, **kw)
    assert every.converged and lazy.converged
    assert every.refreshes == every.steps
    assert 1 <= lazy.refreshes < lazy.steps
    a, b = lazy.state.cpu().numpy(), every.state.cpu().numpy()
    assert np.abs(a - b).max() <= 1e-7 * np.abs(b).max()


def test_eddy_viscosity_drift_is_zero_at_its_reference():
    from aquaflux_gb300 import workloads
    from aquaflux_gb300.refresh import eddy_viscosity, eddy_viscosity_drift

    wl = workloads.channel3d(6, nu=1e-2)
    case = wl.device_case()
    s0 = torch.tensor(wl.initial_state(), device="cuda")
    nut = eddy_viscosity(case, s0)
    assert nut.shape == (case.n_cells,) and bool((nut >= 0).all()) and float(nut.max()) > 0
    drift = eddy_viscosity_drift(case)(s0)
    assert drift(s0) == 0.0
    s1 = s0.clone()
    s1[4 * case.n_cells:5 * case.n_cells] *= 1.5  # k up by half: nu_t moves
    assert drift(s1) > 0.05


def test_reynolds_continuation_reaches_the_direct_root_and_restores_the_viscosity():
    """solve_reynolds_continuation (aquaflux/turbulence/reynolds.py:144-338): the lower-Reynolds
    points change the path, not the root; a point that fails raises and the case keeps its own
    viscosity either way."""
    from aquaflux_gb300 import workloads
    from aquaflux_gb300.solve import newton_solve, reynolds_continuation

    wl = workloads.channel3d(8, renumber=False)
    case = wl.device_case()
    mu0 = case.mu
    direct = newton_solve(case, wl.initial_state(), precision=64, rtol=1e-13, atol=0.0)
    cont = reynolds_continuation(case, wl.initial_state(), 1, precision=64, rtol=1e-13,
                                 atol=0.0)
    assert direct.converged and cont.converged
    assert case.mu == mu0
    assert [p["viscosity_scale"] for p in cont.points] == [10.0, 1.0]
    assert all(p["converged"] for p in cont.points)
    diff = (cont.state - direct.state).abs().max() / direct.state.abs().max()
    assert float(diff) <= 1e-8
    with pytest.raises(RuntimeError, match="point 1 of 2"):
        reynolds_continuation(case, wl.initial_state(), 2, precision=64, max_steps=1,
                              intermediate_rtol=1e-14)
    assert case.mu == mu0
