"""fp32 dual-number passes (``fv_jvp_f32``, ``fv_assemble_jacobian_f32``): the same templates in
single precision agree with the fp64 JVP and Jacobian to fp32 rounding, and a Newton solve whose
linear solves use them reaches the fp64 root (its residual, update and stopping test stay fp64)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from tests.cases import device_case

pytestmark = pytest.mark.gpu

NAMES = ["cav8", "lam3", "sst2", "sst3", "csst3", "lsst2", "wsst2", "bsst3", "psst2"]


def _rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


@pytest.mark.parametrize("name", NAMES)
def test_fp32_jvp_and_assembly_agree_with_fp64(name):
    from aquaflux_gb300.solve import BlockJacobian

    fc, _, d, p = device_case(name)
    s = torch.tensor(d[p + "states"][0], device="cuda")
    rng = np.random.default_rng(11)
    v = torch.tensor(rng.standard_normal(fc.n_unknowns) * (np.abs(d[p + "states"][0]) + 1e-3),
                     device="cuda")
    assert _rel(fc.jvp(s, v, precision=32), fc.jvp(s, v)) <= 2e-4
    j64 = BlockJacobian(fc).materialize(s).clone()
    j32 = BlockJacobian(fc, precision=32).materialize(s).clone()
    fin = torch.isfinite(j64)
    assert torch.equal(fin, torch.isfinite(j32))
    assert _rel(j32[fin], j64[fin]) <= 2e-4


def test_newton_with_fp32_tangents_reaches_the_fp64_root():
    from aquaflux_gb300 import workloads
    from aquaflux_gb300.solve import newton_solve

    wl = workloads.channel3d(12)
    case = wl.device_case()
    a = newton_solve(case, wl.initial_state(), kind="amg", precision=64)
    b = newton_solve(case, wl.initial_state(), kind="amg", precision=32, tangents=32)
    assert a.converged and b.converged
    sa, sb = a.state.cpu().numpy(), b.state.cpu().numpy()
    assert np.abs(sa - sb).max() <= 1e-8 * np.abs(sa).max()
