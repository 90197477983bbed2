"""``torch.autograd.Function`` binding of the residual: forward = ``fv_residual``, backward = the
hand-written adjoints (``fv_vjp`` for the state, ``fv_param_vjp`` for the viscosity and the inlet
scale, ``fv_node_vjp`` for the mesh node coordinates).

The reference differentiates its residual closure with ``jax.vjp`` (``aquaflux/solve/implicit.py:
753-760``); this is the same contract for torch callers::

    R = residual(case, state, mu, inlet_scale, nodes)   # tensors; any may require grad
    (R * w).sum().backward()

``mu`` and ``inlet_scale`` are 0-d tensors (or floats); ``nodes`` (optional) is an
``(n_nodes, dim)`` tensor: when given, the mesh geometry is recomputed from it on the device, and
for a turbulent case the SST wall distance too (to each cell's nearest wall face found at case
creation, held fixed -- the function the mesh-coordinate adjoint differentiates).
"""
from __future__ import annotations

import torch

from ._lib import check, lib, ptr


def _stream() -> int:
    return int(torch.cuda.current_stream().cuda_stream)


class _Residual(torch.autograd.Function):
    @staticmethod
    def forward(ctx, case, state, mu, inlet_scale, nodes):
        s = torch.as_tensor(state, dtype=torch.float64, device="cuda").contiguous()
        case.set_params(mu=float(mu), inlet_scale=float(inlet_scale))
        if nodes is not None:
            case.set_nodes(nodes.detach())
        ctx.case = case
        ctx.has_nodes = nodes is not None
        ctx.devices = (state.device if torch.is_tensor(state) else s.device, mu.device,
                       inlet_scale.device, nodes.device if nodes is not None else None)
        ctx.save_for_backward(s)
        return case.residual(s)

    @staticmethod
    def backward(ctx, w):
        (s,) = ctx.saved_tensors
        case = ctx.case
        w = w.contiguous()
        ds, dm, di, dn = ctx.devices
        gs = case.vjp(s, w).to(ds) if ctx.needs_input_grad[1] else None
        gmu = gsc = None
        if ctx.needs_input_grad[2] or ctx.needs_input_grad[3]:
            p = case.param_vjp(s, w)
            gmu, gsc = p[0].to(dm), p[1].to(di)
        gn = case.node_vjp(s, w).to(dn) if (ctx.has_nodes and ctx.needs_input_grad[4]) else None
        return None, gs, gmu, gsc, gn


def residual(case, state, mu=None, inlet_scale=None, nodes=None) -> torch.Tensor:
    """``R(state; mu, inlet_scale, nodes)`` of a :class:`aquaflux_gb300.fv.FlowCase`, differentiable
    in every tensor argument."""
    mu = torch.as_tensor(case.mu if mu is None else mu, dtype=torch.float64)
    sc = torch.as_tensor(case.inlet_scale if inlet_scale is None else inlet_scale,
                         dtype=torch.float64)
    return _Residual.apply(case, state, mu, sc, nodes)
