"""The premise of the linearised SST closure (``k_lin_closure_coef`` / ``k_closure_lin``): off the
wall, a cell's closure fields (F1, nu_t, the k and omega diffusivities, F2) and its k / omega source
terms depend on the velocity gradient only through the strain rate S, and on grad k, grad omega
only through grad k . grad omega, so their tangents are linear forms in (k', omega', S',
(grad k . grad omega)').  Checked on the oracle's closure (the reference's formulas,
``aquaflux/turbulence/sst.py``, ``sources.py``) with autograd: the gradient of every output with
respect to grad u is a multiple of dS/d(grad u) = 2 s / S, and with respect to grad k (grad omega)
the same multiple of grad omega (grad k)."""
from __future__ import annotations

import numpy as np
import torch

from oracle import fv_oracle as fo


def _off_wall_outputs(gu, k, w, gk, gw, nu, d, vol):
    """The closure of ``Oracle._residual`` off the wall and its k / omega source terms."""
    strain = fo.strain_rate_magnitude(gu)
    f1 = fo.sst_f1(k, w, nu, d, gk, gw)
    nut = fo.sst_nut(k, w, strain, nu, d)
    gam_k = nu + fo.blend(f1, fo.SIGMA_K1, fo.SIGMA_K2) * nut
    gam_w = nu + fo.blend(f1, fo.SIGMA_W1, fo.SIGMA_W2) * nut
    f2 = fo.sst_f2(k, w, nu, d)
    limit = fo.PRODUCTION_LIMIT_RATIO * fo.BETA_STAR * torch.clamp(k, min=0.0) * w
    r_k = -torch.minimum(nut * strain ** 2, limit) * vol + fo.BETA_STAR * k * w * vol
    alpha = fo.blend(f1, fo.ALPHA_1, fo.ALPHA_2)
    beta = fo.blend(f1, fo.BETA_1, fo.BETA_2)
    cap = limit / torch.clamp(nut, min=fo.EDDY_VISCOSITY_FLOOR)
    cross = 2.0 * (1.0 - f1) * fo.SIGMA_W2 * (gk * gw).sum(-1) / w
    r_w = (-alpha * torch.minimum(strain ** 2, cap) * vol + beta * w ** 2 * vol) - cross * vol
    return {"F1": f1, "nu_t": nut, "k diffusivity": gam_k, "omega diffusivity": gam_w, "F2": f2,
            "k source": r_k, "omega source": r_w}


def _residual_off_line(g, direction):
    """|g - c direction| / |g| per cell, c the least-squares multiple (cells where g vanishes
    give 0)."""
    dims = tuple(range(1, g.dim()))
    c = (g * direction).sum(dims) / (direction * direction).sum(dims)
    shape = (-1,) + (1,) * (g.dim() - 1)
    off = (g - c.view(shape) * direction).flatten(1).norm(dim=1)
    scale = g.flatten(1).norm(dim=1)
    return torch.where(scale > 0, off / torch.where(scale > 0, scale, 1.0), 0.0), c


def test_off_wall_closure_tangents_factor_through_four_scalars():
    rng = np.random.default_rng(3)
    n = 4000
    t = lambda a: torch.tensor(a, dtype=torch.float64)  # noqa: E731
    gu = t(rng.standard_normal((n, 3, 3)) * 10.0 ** rng.uniform(-2, 2, (n, 1, 1)))
    k = t(np.where(rng.random(n) < 0.1, 0.0, 10.0 ** rng.uniform(-6, 0, n)))  # some at the clamp
    w = t(10.0 ** rng.uniform(-1, 4, n))
    gk = t(rng.standard_normal((n, 3)) * 10.0 ** rng.uniform(-3, 1, (n, 1)))
    gw = t(rng.standard_normal((n, 3)) * 10.0 ** rng.uniform(-1, 3, (n, 1)))
    nu = t(np.full(n, 5e-4))
    d = t(10.0 ** rng.uniform(-3, -0.3, n))
    vol = t(10.0 ** rng.uniform(-7, -5, n))
    for x in (gu, gk, gw):
        x.requires_grad_(True)
    outs = _off_wall_outputs(gu, k, w, gk, gw, nu, d, vol)
    s = 0.5 * (gu + gu.transpose(-1, -2)).detach()
    strain = fo.strain_rate_magnitude(gu.detach())
    ds_dgu = 2.0 * s / strain[:, None, None]
    branches = 0
    for name, out in outs.items():
        if not out.requires_grad:  # F2: a function of k and omega alone
            continue
        g_u, g_k, g_w = torch.autograd.grad(out.sum(), (gu, gk, gw), allow_unused=True,
                                            retain_graph=True)
        g_u = torch.zeros_like(gu) if g_u is None else g_u
        g_k = torch.zeros_like(gk) if g_k is None else g_k
        g_w = torch.zeros_like(gw) if g_w is None else g_w
        # through S alone
        off, _ = _residual_off_line(g_u, ds_dgu)
        assert float(off.max()) <= 1e-12, name
        # through grad k . grad omega alone: d/d(grad k) = c grad omega, d/d(grad omega) = c grad k
        off_k, c_k = _residual_off_line(g_k, gw.detach())
        off_w, c_w = _residual_off_line(g_w, gk.detach())
        assert float(off_k.max()) <= 1e-12 and float(off_w.max()) <= 1e-12, name
        live = g_k.flatten(1).norm(dim=1) > 0
        assert torch.allclose(c_k[live], c_w[live], rtol=1e-12, atol=0.0), name
        branches += int(live.sum())
    assert branches > 0  # the cross-diffusion branch is exercised, not clipped everywhere


def test_the_check_rejects_an_output_that_reads_one_gradient_entry():
    """A planted dependence on one velocity-gradient entry (not through S) is caught."""
    rng = np.random.default_rng(4)
    gu = torch.tensor(rng.standard_normal((200, 3, 3)), dtype=torch.float64, requires_grad=True)
    strain = fo.strain_rate_magnitude(gu)
    planted = strain ** 2 + 1e-3 * gu[:, 0, 1]
    (g,) = torch.autograd.grad(planted.sum(), gu)
    s = 0.5 * (gu + gu.transpose(-1, -2)).detach()
    off, _ = _residual_off_line(g, 2.0 * s / strain.detach()[:, None, None])
    assert float(off.min()) > 1e-6
