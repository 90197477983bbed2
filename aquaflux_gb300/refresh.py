"""When to rebuild a frozen preconditioner: the reference's staleness triggers.

A march (``pseudo_transient_solve``) or a Newton solve (``newton_solve``) given a trigger
materialises the Jacobian once, then between refreshes only re-forms the preconditioner at each
new shift (the beta-only refresh); after every accepted step it appends a :class:`StepReport` to
the current segment's history and asks the trigger whether to rebuild.

* :class:`CycleGrowthTrigger` -- ``aquaflux/solve/march.py:130-209``: fire when the last
  ``patience`` steps each cost at least ``growth`` times the segment's cheapest measured step,
  past a ``warmup``, and only once the residual has fallen to ``max_residual_ratio`` of the
  reference norm (the developed-flow gate that suppresses the cost rise the shift ramp causes).
* :class:`CoefficientDriftTrigger` -- ``march.py:212-285``: fire once the frozen coefficients have
  drifted by ``threshold`` (relative) since the segment began, past a ``warmup``.
* :func:`eddy_viscosity_drift` -- ``aquaflux/turbulence/coupled.py:681-717``: the drift measure,
  ``||nu_t(state) - nu_t(reference)|| / ||nu_t(reference)||`` with ``nu_t`` from the GPU closure
  (``fv_eddy_viscosity``); re-based at every refresh.

Triggers are pure functions of the history, as in the reference.  The cost signal here is the
accepted step's FGMRES iteration count (the reference reads lineax's step count).
"""
from __future__ import annotations

import dataclasses
from typing import Callable, Sequence

import torch


@dataclasses.dataclass(frozen=True)
class StepReport:
    """What one step cost and where it left the residual (``aquaflux/solve/forward_step.py:219``):
    ``cycles`` the accepted step's Krylov iterations (0 = no measurement), ``residual_ratio`` its
    residual norm over the reference norm, ``drift`` the drift measure (0 without one)."""

    step: int
    cycles: int
    residual_norm: float
    residual_ratio: float
    drift: float = 0.0


@dataclasses.dataclass(frozen=True)
class CycleGrowthTrigger:
    growth: float = 2.0
    max_residual_ratio: float = 5e-2
    warmup: int = 5
    patience: int = 2

    def should_refresh(self, history: Sequence[StepReport]) -> bool:
        if len(history) <= self.warmup or len(history) < self.patience:
            return False
        if history[-1].residual_ratio > self.max_residual_ratio:
            return False
        # zero counts are "no measurement" and never set the baseline
        measured = [r.cycles for r in history if r.cycles > 0]
        if not measured:
            return False
        threshold = self.growth * min(measured)
        return all(r.cycles > 0 and r.cycles >= threshold for r in history[-self.patience:])


@dataclasses.dataclass(frozen=True)
class CoefficientDriftTrigger:
    threshold: float = 0.1
    warmup: int = 3

    def should_refresh(self, history: Sequence[StepReport]) -> bool:
        if len(history) <= self.warmup:
            return False
        return history[-1].drift >= self.threshold


def eddy_viscosity(case, state) -> torch.Tensor:
    """``nu_t`` per cell of a turbulent :class:`aquaflux_gb300.fv.FlowCase` at ``state``."""
    from ._lib import check, lib, ptr

    s = case._vec(state)
    out = torch.empty(case.n_cells, dtype=torch.float64, device="cuda")
    check(lib().fv_eddy_viscosity(case.handle, ptr(s), ptr(out),
                                  int(torch.cuda.current_stream().cuda_stream)))
    return out


def eddy_viscosity_drift(case) -> Callable[[torch.Tensor], Callable[[torch.Tensor], float]]:
    """``reference_state -> (state -> drift)``: the relative ``nu_t`` drift from the state the
    preconditioner was frozen at (the solvers re-base it at every refresh)."""

    def rebase(reference_state):
        ref = eddy_viscosity(case, reference_state).clone()
        scale = max(float(torch.linalg.vector_norm(ref)), torch.finfo(torch.float64).tiny)

        def drift(state) -> float:
            return float(torch.linalg.vector_norm(eddy_viscosity(case, state) - ref)) / scale

        return drift

    return rebase
