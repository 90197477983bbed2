"""GPU Newton-Krylov: materialised Jacobians, ILU(0) preconditioning, converged fields vs the oracle."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import fv_oracle as fo

pytestmark = pytest.mark.gpu

CAVITY_BC = {"top": ("moving", (1.0, 0.0)), "bottom": ("wall",), "left": ("wall",),
             "right": ("wall",)}


def _cavity(n, mu=0.01):
    from aquaflux_gb300 import fv, mesh as fm

    m = fm.structured_grid_2d(n, n)
    return m, fv.FlowCase(fv.DeviceMesh(m), mu=mu, rho=1.0, flow_bc=CAVITY_BC, pressure_pin=0)


@pytest.mark.parametrize("frozen,reach", [(True, 1), (False, 3)])
def test_materialised_jacobian_reproduces_the_operator(frozen, reach):
    from aquaflux_gb300.solve import BlockJacobian

    m, case = _cavity(10)
    rng = np.random.default_rng(0)
    s = torch.tensor(rng.standard_normal(case.n_unknowns) * 0.3, device="cuda")
    jac = BlockJacobian(case, reach=reach, frozen=frozen)
    jac.materialize(s)
    A = jac.to_scipy()
    v = rng.standard_normal(case.n_unknowns)
    n, b = jac.n, jac.b
    v_cm = v.reshape(b, n).T.reshape(-1)
    got = (A @ v_cm).reshape(n, b).T.reshape(-1)
    from aquaflux_gb300._lib import check, lib, ptr

    ref = torch.empty_like(s)
    vv = torch.tensor(v, device="cuda")
    if frozen:
        check(lib().fv_jvp_frozen(case.handle, ptr(s), ptr(vv), ptr(ref),
                                  torch.cuda.current_stream().cuda_stream))
    else:
        ref = case.jvp(s, vv)
    ref = ref.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def _oracle_newton(case_dict, state, steps=20):
    """Dense Newton on the CPU oracle (small cases only)."""
    orc = fo.Oracle(case_dict)
    x = torch.as_tensor(state, dtype=torch.float64).clone()
    for _ in range(steps):
        r = orc.residual(x)
        if float(torch.linalg.vector_norm(r)) < 1e-13:
            break
        J = torch.autograd.functional.jacobian(orc.residual, x)
        x = x - torch.linalg.solve(J, r)
    return x.numpy(), float(torch.linalg.vector_norm(orc.residual(x)))


@pytest.mark.parametrize("precision", [64, 32])
def test_newton_cavity_converges_to_the_oracle_root(precision):
    from aquaflux_gb300.solve import newton_solve

    m, case = _cavity(16)
    res = newton_solve(case, np.zeros(case.n_unknowns), precision=precision, max_steps=30)
    assert res.converged, res.residual_norms
    s = res.state.cpu().numpy()
    cd = fo.make_case(m, mu=0.01, rho=1.0, flow_bc=CAVITY_BC, pressure_pin=0)
    ref, ref_norm = _oracle_newton(cd, s)
    assert ref_norm < 1e-12
    assert np.abs(s - ref).max() <= 1e-8 * np.abs(ref).max()
    r_oracle = fo.Oracle(cd).residual(torch.as_tensor(s)).numpy()
    assert np.linalg.norm(r_oracle) <= 1e-12 + 1e-10 * res.residual_norms[0]


def test_fp32_and_fp64_preconditioners_reach_the_same_root():
    from aquaflux_gb300.solve import newton_solve

    m, case = _cavity(24)
    a = newton_solve(case, np.zeros(case.n_unknowns), precision=64)
    b = newton_solve(case, np.zeros(case.n_unknowns), precision=32)
    assert a.converged and b.converged
    sa, sb = a.state.cpu().numpy(), b.state.cpu().numpy()
    assert np.abs(sa - sb).max() <= 1e-8 * np.abs(sa).max()


def test_implicit_adjoint_matches_finite_differences_of_the_solve():
    """d(mean |u|)/d mu through the converged cavity, against central differences of the solve
    (the check of the reference's tests/integration/test_cavity.py:74-95)."""
    from aquaflux_gb300.solve import implicit_adjoint, newton_solve

    n = 12
    m, case = _cavity(n)
    z = np.zeros(case.n_unknowns)

    def mean_speed(mu):
        case.set_params(mu=mu)
        res = newton_solve(case, z, precision=64, max_steps=40, reach=3, frozen=False, rtol=1e-14)
        assert res.converged
        u = res.state[: n * n]
        return float(u.abs().mean()), res.state

    mu0 = 0.01
    f0, state = mean_speed(mu0)
    u = state[: n * n]
    g = torch.zeros_like(state)
    g[: n * n] = torch.sign(u) / (n * n)
    case.set_params(mu=mu0)
    adj = implicit_adjoint(case, state, g)
    assert adj.converged
    h = 1e-5
    fd = (mean_speed(mu0 + h)[0] - mean_speed(mu0 - h)[0]) / (2 * h)
    case.set_params(mu=mu0)
    grad = float(adj.dparams[0])
    assert abs(fd) > 1e-3
    assert abs(grad - fd) <= 1e-4 * abs(fd)


@pytest.mark.parametrize("precision,fine_order", [(32, "natural"), (64, "natural"),
                                                  (32, "colour")])
def test_amg_vcycle_is_a_fixed_linear_operator_and_converges_newton(precision, fine_order):
    """The V-cycle is fixed-linear (tests/unit/test_host_vcycle.py:76) and, as the FGMRES
    preconditioner, drives the SST channel's Newton solve to the same root as ILU(0)."""
    from aquaflux_gb300 import workloads
    from aquaflux_gb300.amg import AmgPreconditioner
    from aquaflux_gb300.solve import BlockJacobian, newton_solve

    wl = workloads.channel3d(16)
    case = wl.device_case()
    jac = BlockJacobian(case)
    pc = AmgPreconditioner(jac, precision, fine_order=fine_order, min_cells=200)
    assert len(pc.h.levels) >= 2
    s = torch.tensor(wl.initial_state(), device="cuda")
    pc.refresh(s)
    r1 = torch.randn(case.n_unknowns, dtype=torch.float64, device="cuda")
    r2 = torch.randn_like(r1)
    a = pc.apply(r1).clone()
    b = pc.apply(r2).clone()
    ab = pc.apply(2.0 * r1 - 3.0 * r2).clone()
    tol = 1e-4 if precision == 32 else 1e-11
    assert float((ab - (2.0 * a - 3.0 * b)).abs().max()) <= tol * float(ab.abs().max())
    res_amg = newton_solve(case, wl.initial_state(), kind="amg", precision=precision,
                           precond_options={"fine_order": fine_order}, max_steps=40)
    res_ilu = newton_solve(case, wl.initial_state(), precision=64, max_steps=40)
    assert res_amg.converged and res_ilu.converged
    sa, si = res_amg.state.cpu().numpy(), res_ilu.state.cpu().numpy()
    assert np.abs(sa - si).max() <= 1e-7 * np.abs(si).max()


@pytest.mark.parametrize("name", ["cav8", "cavj", "lam3", "sst2", "sst3", "ccavj", "csst3", "lcavj",
                                  "lsst2", "wsst2", "bsst3", "psst2", "msst2"])
def test_assembled_jacobian_equals_the_coloured_probe(name):
    """The direct face assembly of J_direct gives the blocks the coloured probes of the frozen JVP
    give (materialize_block_jacobian, aquaflux/solve/sparse_jacobian.py:722-847), at the golden
    states (negative-k cells, wall cells, the pressure pin) and at the zero state (mass-flux ties)."""
    from tests.cases import device_case

    from aquaflux_gb300.solve import BlockJacobian

    fc, _, d, p = device_case(name)
    ja = BlockJacobian(fc, method="assemble")
    jp = BlockJacobian(fc, method="probe")
    states = [np.asarray(x) for x in d[p + "states"]] + [np.zeros(fc.n_unknowns)]
    for st in states:
        s = torch.tensor(st, device="cuda")
        a = ja.materialize(s).clone()
        b = jp.materialize(s).clone()
        # omega = 0 (the SST zero state) makes both operators non-finite at the same entries
        assert torch.equal(torch.isfinite(a), torch.isfinite(b)), name
        fin = torch.isfinite(b)
        scale = float(b[fin].abs().max())
        assert float((a[fin] - b[fin]).abs().max()) <= 1e-14 * scale, name


def test_assembled_jacobian_overwrites_stale_values():
    """Every block of the pattern is rewritten (no accumulation into what the buffer held)."""
    from aquaflux_gb300.solve import BlockJacobian

    m, case = _cavity(6)
    jac = BlockJacobian(case)
    s = torch.tensor(np.random.default_rng(3).standard_normal(case.n_unknowns) * 0.2,
                     device="cuda")
    a = jac.materialize(s).clone()
    jac.values.fill_(7.0)
    b = jac.materialize(s)
    assert torch.equal(a, b)


@pytest.fixture(scope="module")
def cavity64_solves():
    """Config 1: the 64 x 64 lid-driven cavity (Re = 100), solved from the zero state on the GPU
    with the fp64 and the fp32-preconditioned forms (ILU(0) and AMG): to the reference's
    tolerance (1e-10 relative), and on to the root (1e-13 relative)."""
    from aquaflux_gb300.solve import newton_solve

    m, case = _cavity(64)
    out = {}
    for kind, prec in (("ilu", 64), ("ilu", 32), ("amg", 32)):
        for rtol in (1e-10, 1e-13):
            out[(kind, prec, rtol)] = newton_solve(case, np.zeros(case.n_unknowns), kind=kind,
                                                   precision=prec, rtol=rtol, atol=0.0,
                                                   max_steps=60)
    return m, out


def test_config1_cavity_64_newton_meets_the_oracle_residual(cavity64_solves):
    """Every form stops at the reference's tolerance on the oracle's own residual:
    ||R_oracle(s)|| <= 1e-12 + 1e-10 ||R_oracle(0)||."""
    m, out = cavity64_solves
    cd = fo.make_case(m, mu=0.01, rho=1.0, flow_bc=CAVITY_BC, pressure_pin=0)
    orc = fo.Oracle(cd)
    r0 = float(np.linalg.norm(orc.residual(torch.zeros(3 * 64 * 64, dtype=torch.float64))))
    for key, res in out.items():
        if key[2] != 1e-10:
            continue
        assert res.converged, (key, res.residual_norms)
        r = orc.residual(torch.as_tensor(res.state.cpu().numpy())).numpy()
        assert np.linalg.norm(r) <= 1e-12 + 1e-10 * r0, key


def test_config1_cavity_64_newton_matches_an_independent_root(cavity64_solves):
    """The converged fields against an independent FP64 root: the oracle's Newton with the exact
    sparse Jacobian (reverse-mode products of the oracle) and sparse LU solves, from the zero
    state to the oracle's round-off.  Every GPU form solved on to 1e-13 relative matches it to
    1e-8; at the reference's 1e-10 the fields are within what that tolerance allows on this
    operator (the pressure, pinned in one cell, moves most), 1e-6."""
    from oracle.newton_oracle import OracleJacobian, newton

    m, out = cavity64_solves
    cd = fo.make_case(m, mu=0.01, rho=1.0, flow_bc=CAVITY_BC, pressure_pin=0)
    orc = fo.Oracle(cd)
    jac = OracleJacobian(orc, m.owner, m.neighbour, 64 * 64, 3)
    ref = newton(orc, jac, np.zeros(3 * 64 * 64), rtol=1e-15, atol=0.0, max_steps=12)
    root = ref["state"]
    assert ref["residual_norms"][-1] <= 1e-14 * ref["residual_norms"][0]
    for key, res in out.items():
        s = res.state.cpu().numpy()
        bound = 1e-8 if key[2] == 1e-13 else 1e-6
        assert np.abs(s - root).max() <= bound * np.abs(root).max(), key
