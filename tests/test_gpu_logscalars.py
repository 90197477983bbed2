"""Log-solved turbulence scalars (``LogScalars``, ``aquaflux/turbulence/coupled.py:178-207``) on the
GPU: the same root as the direct parametrisation, omega > 0 along the whole solve by construction,
the near-wall omega rows linear in the solved variable, and the IFT adjoint unchanged at the root."""
from __future__ import annotations

import dataclasses

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = b.detach().cpu().numpy() if torch.is_tensor(b) else np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def wl_cells(wl):
    return wl.mesh.n_cells


def _channel(**kw):
    from aquaflux_gb300 import workloads

    wl = workloads.channel3d(12, 8, 8)
    return dataclasses.replace(wl, **kw)


def test_log_omega_newton_reaches_the_direct_root():
    """The productive combination (direct k, log omega, ``CoupledRANS.build`` docstring,
    coupled.py:322-324).  A log k is covered at the operator level (residual, JVP, VJP, Jacobian
    assembly against the reference's goldens): Newton in log k from a uniform inlet k drives the
    near-wall k of this channel below the double range in its first steps."""
    from aquaflux_gb300.solve import newton_solve

    direct = _channel()
    logw = _channel(omega_transform="log")
    fd, fl = direct.device_case(), logw.device_case()
    s0 = direct.initial_state()
    a = newton_solve(fd, s0, precision=64, max_steps=40)
    b = newton_solve(fl, fl.to_solved(s0), precision=64, max_steps=40)
    assert a.converged and b.converged
    assert _rel(fl.to_physical(b.state), a.state) <= 1e-8
    # converged to the solver's criterion on the log case's own residual (physical transport
    # rows, log-ratio wall rows), and omega > 0 by construction
    assert float(torch.linalg.vector_norm(fl.residual(b.state))) <= \
        1e-10 * b.residual_norms[0] + 1e-12
    assert bool((fl.to_physical(b.state)[-wl_cells(logw):] > 0).all())


def test_wall_rows_are_linear_in_log_omega():
    """LogRatioRow: R_w = log(omega / omega_wall) = w - log(omega_wall) on the wall cells, so one
    Newton correction on w alone fixes them exactly (fixed_value.py:96-120)."""
    wl = _channel(omega_transform="log")
    fc = wl.device_case()
    s = torch.tensor(fc.to_solved(wl.initial_state(noise=0.05)), device="cuda")
    r = fc.residual(s)
    n, d = wl.mesh.n_cells, wl.mesh.dim
    wall = torch.zeros(n, dtype=torch.bool, device="cuda")
    owners = np.concatenate([wl.mesh.owner[wl.mesh.patches[p]] for p in wl.sst["walls"]])
    wall[torch.as_tensor(np.unique(owners), device="cuda")] = True
    wrow = slice((d + 2) * n, (d + 3) * n)
    # d R_w / d w = 1 on the wall rows: a shift of w by delta moves them by exactly delta
    delta = torch.zeros_like(s)
    delta[wrow] = torch.where(wall, 0.25, 0.0).to(torch.float64)
    r2 = fc.residual(s + delta)
    assert float((r2[wrow][wall] - r[wrow][wall] - 0.25).abs().max()) <= 1e-12
    jv = fc.jvp(s, delta)
    assert float((jv[wrow][wall] - 0.25).abs().max()) <= 1e-12


def test_adjoint_gradient_is_invariant_under_the_transform():
    """At the root the IFT gradient of a flux functional does not depend on the parametrisation
    (the realizability floor is inactive there)."""
    from aquaflux_gb300.solve import functional_gradient, newton_solve

    out = []
    for tr in ("direct", "log"):
        wl = _channel(omega_transform=tr)
        fc = wl.device_case()
        res = newton_solve(fc, fc.to_solved(wl.initial_state()), precision=64, rtol=1e-13,
                           atol=1e-14, max_steps=60)
        assert res.converged
        w = fc.functional_weights({"right": {wl.mesh.dim: 1.0}})  # outlet mass flux
        out.append(functional_gradient(fc, res.state, w, nodes=False, rtol=1e-12))
    a, b = out
    assert abs(float(a.value) - float(b.value)) <= 1e-9 * abs(float(a.value))
    assert _rel(b.dparams, a.dparams) <= 1e-6
