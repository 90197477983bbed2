"""The linearised JVP (``fv_linearise`` + ``fv_jvp_linearised``: the interior faces' flux tangents
from the face intermediates a held residual evaluation kept) against the dual-number JVP, on every
first-order-upwind reference case; its refusals; Newton on it."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from cases import device_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["cav8", "cavj", "lam3", "sst2", "sst3", "ccavj", "csst2",
                                  "csst3", "wsst2", "bsst3"])
def test_linearised_jvp_equals_the_dual_number_jvp(name):
    fc, case, d, p = device_case(name)
    rng = np.random.default_rng(13)
    for s in d[p + "states"][:2]:
        v = rng.standard_normal(s.size)
        r = fc.linearise(s)
        assert torch.equal(r, fc.residual(s))  # the same evaluation, intermediates kept
        got = fc.jvp_linearised(s, v)
        ref = fc.jvp(s, v)
        scale = float(ref.abs().max())
        assert float((got - ref).abs().max()) <= 1e-12 * scale
        # bitwise run to run
        assert torch.equal(got, fc.jvp_linearised(s, v))


def test_linearised_jvp_refusals():
    from aquaflux_gb300._lib import FvError

    fc, case, d, p = device_case("lcavj")  # limited reconstruction
    s = d[p + "states"][0]
    with pytest.raises(FvError):
        fc.linearise(s)
    fc, case, d, p = device_case("sst2")
    s = d[p + "states"][0]
    v = np.ones(s.size)
    with pytest.raises(FvError):  # nothing held yet
        fc.jvp_linearised(s, v)
    fc.linearise(s)
    fc.jvp_linearised(s, v)
    fc.set_params(mu=fc.mu * 1.1)  # a parameter change drops the linearisation
    with pytest.raises(FvError):
        fc.jvp_linearised(s, v)
    fc.linearise(s)
    assert float((fc.jvp_linearised(s, v) - fc.jvp(s, v)).abs().max()) <= \
        1e-12 * float(fc.jvp(s, v).abs().max())


def test_newton_on_the_linearised_jvp_reaches_the_dual_number_root():
    from aquaflux_gb300 import workloads
    from aquaflux_gb300.solve import newton_solve

    wl = workloads.channel3d(10, renumber="host")
    case = wl.device_case()
    a = newton_solve(case, wl.initial_state(), kind="amg", precision=32, linearised=True,
                     rtol=1e-12)
    b = newton_solve(case, wl.initial_state(), kind="amg", precision=32, linearised=False,
                     rtol=1e-12)
    assert a.converged and b.converged and a.steps == b.steps
    diff = (a.state - b.state).abs().max() / b.state.abs().max()
    assert float(diff) <= 1e-9
