"""Products at a held evaluation: the linearised JVP (``fv_linearise`` + ``fv_jvp_linearised``:
tangent-only flux, coefficient and gradient stages from the intermediates a held residual
evaluation kept) against the dual-number JVP on every first-order-upwind reference case, and the
held-forward VJP (``fv_hold_forward`` + ``fv_vjp_held``) bitwise against ``fv_vjp``; their
refusals; Newton and the IFT adjoint on them."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from cases import device_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["cav8", "cavj", "lam3", "sst2", "sst3", "ccavj", "csst2",
                                  "csst3", "wsst2", "bsst3"])
def test_linearised_jvp_equals_the_dual_number_jvp(name):
    from aquaflux_gb300._lib import check, lib, ptr

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
        # field by field too: the k and omega rows (off-wall closure and source tangents from
        # the tabulated forms) against their own scale
        nf = got.numel() // fc.n_cells
        for q, (a, b) in enumerate(zip(got.view(nf, -1), ref.view(nf, -1))):
            assert float((a - b).abs().max()) <= 1e-11 * float(b.abs().max()) + 1e-300, (name, q)
        # bitwise run to run; with a residual asked for, the held one and the same product
        assert torch.equal(got, fc.jvp_linearised(s, v))
        sv, vv = fc._vec(s), fc._vec(v)
        rr, jv = torch.empty_like(r), torch.empty_like(r)
        check(lib().fv_jvp_linearised(fc._h, ptr(sv), ptr(vv), ptr(rr), ptr(jv),
                                      torch.cuda.current_stream().cuda_stream))
        assert torch.equal(rr, r) and torch.equal(jv, got)


def test_linearised_sst_channel_with_wall_and_off_wall_cells():
    """The 3D SST channel at a perturbed state (wall-function cells beside the walls, off-wall
    cells inside, k clipped at zero in some cells): the linearised product, whose off-wall closure
    and source tangents come from the forms tabulated at the linearisation, against the dual-number
    JVP field by field; and again after a second linearisation at another state."""
    from aquaflux_gb300 import workloads

    wl = workloads.channel3d(8, renumber="host")
    fc = wl.device_case()
    rng = np.random.default_rng(21)
    n = fc.n_cells
    for seed in (0, 1):
        s = wl.initial_state(seed=seed, noise=0.05 + 0.05 * seed)
        s[4 * n:4 * n + n // 10] = 0.0  # k exactly at the clamp (the tie rule) in a tenth of cells
        v = rng.standard_normal(s.size)
        fc.linearise(s)
        got, ref = fc.jvp_linearised(s, v), fc.jvp(s, v)
        for q, (a, b) in enumerate(zip(got.view(6, -1), ref.view(6, -1))):
            assert float((a - b).abs().max()) <= 1e-11 * float(b.abs().max()), q


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


@pytest.mark.parametrize("name", ["cavj", "lam3", "sst3", "csst3", "lcavj", "bsst3", "psst2"])
def test_held_forward_vjp_is_bitwise_the_vjp(name):
    """fv_hold_forward + fv_vjp_held: the adjoint stages alone on the held forward pass give
    bitwise fv_vjp's product (every scheme: corrected gradients, limited reconstruction, log
    scalars), repeatedly."""
    from aquaflux_gb300._lib import FvError

    fc, case, d, p = device_case(name)
    s = d[p + "states"][0]
    rng = np.random.default_rng(17)
    r = fc.hold_forward(s)
    assert torch.equal(r, fc.residual(s))
    with pytest.raises(FvError):  # the residual evaluation dropped the hold
        fc.vjp_held(s, np.ones(s.size))
    fc.hold_forward(s)
    for _ in range(2):
        w = rng.standard_normal(s.size)
        got = fc.vjp_held(s, w)
        assert torch.equal(got, fc.vjp(s, w))  # fv_vjp leaves its forward pass held


def test_held_forward_refusals():
    from aquaflux_gb300._lib import FvError

    fc, case, d, p = device_case("sst2")
    s = d[p + "states"][0]
    w = np.ones(s.size)
    with pytest.raises(FvError):  # nothing held yet
        fc.vjp_held(s, w)
    fc.hold_forward(s)
    fc.vjp_held(s, w)
    fc.jvp(s, w)  # another evaluation overwrites the held pass
    with pytest.raises(FvError):
        fc.vjp_held(s, w)
    fc.hold_forward(s)
    fc.set_params(mu=fc.mu * 1.1)
    with pytest.raises(FvError):
        fc.vjp_held(s, w)


def test_implicit_adjoint_on_the_held_forward_pass():
    """The IFT adjoint solve (now on the held forward pass) equals FGMRES on plain VJPs bitwise."""
    from aquaflux_gb300 import workloads
    from aquaflux_gb300.solve import (BlockJacobian, IluPreconditioner, TransposedPreconditioner,
                                      fgmres, implicit_adjoint, newton_solve)

    wl = workloads.channel3d(8, renumber=False)
    case = wl.device_case()
    root = newton_solve(case, wl.initial_state(), precision=64, rtol=1e-12).state
    g = torch.randn(case.n_unknowns, dtype=torch.float64, device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(5))
    a = implicit_adjoint(case, root, g, rtol=1e-10)
    pc = IluPreconditioner(BlockJacobian(case, reach=1, frozen=True), 64)
    pc.refresh(root)
    b = fgmres(lambda w: case.vjp(root, w), g, TransposedPreconditioner(pc).apply, rtol=1e-10,
               restart=30, maxiter=1000)
    assert a.converged and a.krylov_iterations == b.iterations
    assert torch.equal(a.lam, b.x)


def test_implicit_adjoint_holds_again_after_a_preconditioner_evaluates_the_case():
    """A preconditioner of the caller's that evaluates the residual in every application drops the
    held forward pass each time: the adjoint solve holds it again and gives bitwise the same
    result."""
    from aquaflux_gb300 import workloads
    from aquaflux_gb300.solve import (BlockJacobian, IluPreconditioner, implicit_adjoint,
                                      newton_solve)

    wl = workloads.channel3d(8, renumber=False)
    case = wl.device_case()
    root = newton_solve(case, wl.initial_state(), precision=64, rtol=1e-12).state
    g = torch.randn(case.n_unknowns, dtype=torch.float64, device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(5))

    class Evaluating:
        def __init__(self):
            self.pc = IluPreconditioner(BlockJacobian(case, reach=1, frozen=True), 64)
            self.applications = 0

        def refresh(self, s):
            self.pc.refresh(s)

        def apply_transpose(self, r):
            self.applications += 1
            case.residual(root)  # drops the held forward pass
            return self.pc.apply_transpose(r)

    ev = Evaluating()
    a = implicit_adjoint(case, root, g, rtol=1e-10, preconditioner=ev)
    b = implicit_adjoint(case, root, g, rtol=1e-10)
    assert ev.applications > 1
    assert a.converged and a.krylov_iterations == b.krylov_iterations
    assert torch.equal(a.lam, b.lam)
