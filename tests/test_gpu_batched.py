"""The batched calibration sweep on the GPU: the disjoint-union case reproduces each instance's own
residual, and the per-instance gradients from one adjoint solve match finite differences of
re-converged solves."""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _small():
    from aquaflux_gb300 import workloads

    return workloads.batched_channels(4, n_min=6, n_max=12, seed=3)


def test_union_residual_equals_each_instance():
    from aquaflux_gb300 import fv
    from aquaflux_gb300 import mesh as fm

    bw = _small()
    case = bw.workload.device_case()
    s = bw.initial_state() * (1.0 + 0.1 * np.random.default_rng(0).standard_normal(case.n_unknowns))
    r = case.residual(s).cpu().numpy().reshape(3, -1)
    S = s.reshape(3, -1)
    for i in range(bw.n_instances):
        lo, hi = bw.offsets[i], bw.offsets[i + 1]
        m = fm.structured_grid_2d(int(bw.sizes[i]), int(bw.sizes[i]), 2.0, 1.0)
        ci = fv.FlowCase(fv.DeviceMesh(m), mu=float(bw.mu[i]), rho=1.0,
                         flow_bc={"left": ("inlet", (float(bw.velocity[i]), 0.0)),
                                  "right": ("outlet", 0.0), "bottom": ("wall",),
                                  "top": ("wall",)})
        ri = ci.residual(S[:, lo:hi].reshape(-1)).cpu().numpy().reshape(3, -1)
        assert np.abs(ri - r[:, lo:hi]).max() <= 1e-13 * max(np.abs(ri).max(), 1.0)


def _solve(bw, mu=None, vel=None):
    from aquaflux_gb300 import workloads
    from aquaflux_gb300.solve import newton_solve

    wl = bw.workload
    if mu is not None or vel is not None:
        mu = bw.mu if mu is None else mu
        vel = bw.velocity if vel is None else vel
        flow_bc = dict(wl.flow_bc)
        for i in range(bw.n_instances):
            flow_bc[f"{i}:left"] = ("inlet", (float(vel[i]), 0.0))
        wl = workloads.Workload(wl.name, wl.mesh, np.repeat(mu, np.diff(bw.offsets)), 1.0,
                                flow_bc, None, None)
    case = wl.device_case()
    res = newton_solve(case, bw.initial_state(), precision=64, rtol=1e-13, atol=1e-14,
                       max_steps=60)
    assert res.converged
    return case, res.state


def test_batched_gradients_match_finite_differences():
    from aquaflux_gb300.solve import batched_gradients

    bw = _small()
    case, s = _solve(bw)
    g = batched_gradients(case, s, bw, rtol=1e-13)
    k = 2
    h = 1e-5

    def J(mu=None, vel=None):
        c, st = _solve(bw, mu, vel)
        return batched_gradients(c, st, bw).value.cpu().numpy()

    mu_p, mu_m = bw.mu.copy(), bw.mu.copy()
    mu_p[k] *= 1 + h
    mu_m[k] *= 1 - h
    jp, jm = J(mu=mu_p), J(mu=mu_m)
    fd = (jp - jm) / (2 * h * bw.mu[k])
    assert abs(float(g.dmu[k]) - fd[k]) <= 1e-5 * max(abs(fd[k]), 1e-6)
    others = np.delete(np.arange(bw.n_instances), k)
    assert np.abs(jp[others] - jm[others]).max() <= 1e-12  # instances are independent
    v_p, v_m = bw.velocity.copy(), bw.velocity.copy()
    v_p[k] += h
    v_m[k] -= h
    fd = (J(vel=v_p)[k] - J(vel=v_m)[k]) / (2 * h)
    assert abs(float(g.dvelocity[k]) - fd) <= 1e-5 * max(abs(fd), 1e-6)


def test_autotune_keeps_results_bitwise():
    bw = _small()
    case = bw.workload.device_case()
    s = bw.initial_state()
    w = np.random.default_rng(1).standard_normal(case.n_unknowns)
    ref = case.vjp(s, w)
    best = case.autotune(s, w)
    assert best in (32, 64, 96, 128)
    for tb in (32, 64, 128):
        case.set_block_size(tb)
        assert torch.equal(case.vjp(s, w), ref)


@pytest.mark.parametrize("which", ["batched", "sst_channel"])
def test_persistent_launch_is_bitwise_the_stage_launches(which):
    """Residual + VJP as one persistent cooperative launch (every stage in one kernel, grid-wide
    barriers between them) equals the stage-per-launch evaluation bit for bit, for every block size
    and chunk the autotuner tries, on the batched instances and on an SST channel."""
    from aquaflux_gb300 import workloads

    if which == "batched":
        bw = _small()
        case = bw.workload.device_case()
        s = torch.tensor(bw.initial_state(), device="cuda")
    else:
        wl = workloads.channel3d(10)
        case = wl.device_case()
        s = torch.tensor(wl.initial_state(noise=0.05), device="cuda")
    w = torch.randn(case.n_unknowns, dtype=torch.float64, device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(1))
    r0, g0 = case.vjp(s, w, return_residual=True)
    for block in (64, 128):
        for chunk in (1, 2, 4, 8):
            case.set_persistent(True, block, chunk)
            r1, g1 = case.vjp(s, w, return_residual=True)
            assert torch.equal(r1, r0) and torch.equal(g1, g0), (block, chunk)
    case.set_persistent(False)
    block, chunk, ms = case.autotune_persistent(s, w)
    assert block in (64, 128) and chunk in (1, 2, 4, 8) and ms > 0
    r2, g2 = case.vjp(s, w, return_residual=True)  # the tuner leaves the path off
    assert torch.equal(g2, g0)
