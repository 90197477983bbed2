"""The backward-facing-step configuration (2D, coupled u, v, p + k-omega SST at Re_h = 5e4,
corrected Green-Gauss gradients on a graded, jittered two-block quad mesh): residual, JVP and VJP
against the oracle and central differences (step 1e-7), at fixture size and at the full ~200k
cells."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import fv_oracle as fo
from tests.cases import workload_oracle_case

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = b.detach().cpu().numpy() if torch.is_tensor(b) else np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _setup(**kw):
    from aquaflux_gb300 import workloads

    wl = workloads.backward_step(**kw)
    return wl, wl.device_case(), fo.Oracle(workload_oracle_case(wl))


@pytest.mark.parametrize("size", ["small", "full"])
def test_backward_step_residual_jvp_vjp_match_oracle(size):
    kw = dict(n_step=6, n_channel=8, n_upstream=6, n_downstream=20) if size == "small" else {}
    wl, fc, orc = _setup(**kw)
    s = wl.initial_state(noise=0.05)
    assert _rel(fc.residual(s), orc.residual(torch.as_tensor(s))) <= 1e-12
    rng = np.random.default_rng(5)
    v = rng.standard_normal(s.size) * (np.abs(s) + 1e-3)
    assert _rel(fc.jvp(s, v), orc.jvp(s, v)) <= 1e-11
    w = rng.standard_normal(s.size)
    assert _rel(fc.vjp(s, w), orc.vjp(s, w)) <= 1e-11


def test_backward_step_jvp_matches_central_differences():
    """J v against (R(s + h v) - R(s - h v)) / 2h with h = 1e-7, both residuals on the GPU."""
    wl, fc, _ = _setup()
    s = wl.initial_state(noise=0.05)
    rng = np.random.default_rng(7)
    v = rng.standard_normal(s.size) * (np.abs(s) + 1e-3)
    h = 1e-7
    fd = (fc.residual(s + h * v) - fc.residual(s - h * v)) / (2 * h)
    assert _rel(fc.jvp(s, v), fd) <= 1e-6
