"""Shifted / equilibrated cell-major operators, exact preconditioner transposes and batched JVPs on
the GPU."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import operator_oracle as oo
from tests.cases import golden

pytestmark = pytest.mark.gpu


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _run_shift_equilibrate(d, shift, equilibrate, out_f64=True):
    from aquaflux_gb300._lib import check, lib, ptr

    ip = torch.tensor(d["op_bsr_indptr"], device="cuda")
    ix = torch.tensor(d["op_bsr_indices"], device="cuda")
    blocks = torch.tensor(d["op_blocks"].reshape(-1), device="cuda")
    n, b = len(d["op_bsr_indptr"]) - 1, d["op_blocks"].shape[1]
    sh = None if shift is None else torch.tensor(shift, device="cuda")
    scale = torch.empty(n * b, dtype=torch.float64, device="cuda")
    work = torch.empty(2 * n * b + 1, dtype=torch.float64, device="cuda")
    out = torch.empty(blocks.numel(), dtype=torch.float64 if out_f64 else torch.float32,
                      device="cuda")
    check(lib().fv_bsr_shift_equilibrate(n, b, ptr(ip), ptr(ix), ptr(blocks), ptr(sh),
                                         int(equilibrate), ptr(scale), ptr(work), ptr(out),
                                         int(out_f64), _stream()))
    return out.cpu().numpy().reshape(-1, b, b), scale.cpu().numpy()


@pytest.mark.parametrize("shifted,equilibrate", [(True, True), (False, True), (True, False)])
def test_shift_equilibrate_matches_reference_bitwise(shifted, equilibrate):
    d = golden("operator")
    shift = d["op_shift"] if shifted else None
    got, scale = _run_shift_equilibrate(d, shift, equilibrate)
    ref, ref_scale = oo.shift_equilibrate(d["op_blocks"], d["op_bsr_indptr"], d["op_bsr_indices"],
                                          shift, equilibrate)
    assert np.array_equal(got, ref)
    if equilibrate:
        assert np.array_equal(scale, ref_scale)
        key = "op_cm_data" if shifted else "op_eq_cm_data"
        data = oo.bsr_to_cell_major_csr_data(got, d["op_bsr_indptr"], d["op_bsr_indices"])
        assert np.array_equal(data, d[key])


def test_shift_equilibrate_fp32_output_is_the_rounded_fp64():
    d = golden("operator")
    got32, _ = _run_shift_equilibrate(d, d["op_shift"], True, out_f64=False)
    got64, _ = _run_shift_equilibrate(d, d["op_shift"], True)
    assert np.array_equal(got32, got64.astype(np.float32))


def _cavity_pc(kind, precision, **kw):
    from aquaflux_gb300 import workloads
    from aquaflux_gb300.amg import AmgPreconditioner
    from aquaflux_gb300.solve import BlockJacobian, IluPreconditioner

    wl = workloads.channel3d(12)
    case = wl.device_case()
    jac = BlockJacobian(case)
    if kind == "ilu":
        pc = IluPreconditioner(jac, precision, **kw)
    else:
        pc = AmgPreconditioner(jac, precision, min_cells=150, **kw)
    s = torch.tensor(wl.initial_state(noise=0.02), device="cuda")
    return wl, case, pc, s


@pytest.mark.parametrize("kind,opts", [
    ("ilu", {}), ("ilu", {"equilibrate": True}), ("amg", {}),
    ("amg", {"fine_order": "colour"}), ("amg", {"equilibrate": True})])
def test_preconditioner_transpose_is_exact(kind, opts):
    """<M x, y> = <x, M^T y> for the fp64 ILU(0) solve and the fp64 V-cycle (the adjoint
    preconditioner of aquaflux/solve/implicit.py:709-730)."""
    wl, case, pc, s = _cavity_pc(kind, 64, **opts)
    shift = torch.rand(case.n_unknowns, dtype=torch.float64, device="cuda")
    pc.shift = shift if kind == "ilu" and opts else pc.shift
    pc.refresh(s)
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn(case.n_unknowns, dtype=torch.float64, device="cuda", generator=g)
    y = torch.randn(case.n_unknowns, dtype=torch.float64, device="cuda", generator=g)
    lhs = float(torch.dot(pc.apply(x), y))
    rhs = float(torch.dot(x, pc.apply_transpose(y)))
    assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), 1.0)


@pytest.mark.parametrize("precision,fine_order", [(32, "colour"), (32, "natural"),
                                                  (64, "natural"), (64, "colour")])
def test_graph_replayed_vcycle_equals_the_eager_cycle(precision, fine_order):
    """The V-cycle and its transpose, each replayed as one CUDA graph, give bitwise the eager
    cycle's output: on the first (eager) and second (captured) application, after a refresh at a
    new state, and after a new shift (which re-forms the fine operator's storage and so
    re-captures)."""
    _, case, pg, s = _cavity_pc("amg", precision, fine_order=fine_order)
    _, _, pe, _ = _cavity_pc("amg", precision, fine_order=fine_order, graph=False)
    g = torch.Generator(device="cuda").manual_seed(1)
    rs = [torch.randn(case.n_unknowns, dtype=torch.float64, device="cuda", generator=g)
          for _ in range(3)]
    for p in (pg, pe):
        p.refresh(s)
    for r in rs:
        assert torch.equal(pg.apply(r), pe.apply(r))
        assert torch.equal(pg.apply_transpose(r), pe.apply_transpose(r))
    assert set(pg._graphs) == {False, True}
    s2 = s * (1.0 + 0.01 * torch.rand(s.shape, dtype=s.dtype, device="cuda", generator=g))
    for p in (pg, pe):
        p.refresh(s2)
    for r in rs:
        assert torch.equal(pg.apply(r), pe.apply(r))
        assert torch.equal(pg.apply_transpose(r), pe.apply_transpose(r))
    shift = 0.5 + torch.rand(case.n_unknowns, dtype=torch.float64, device="cuda", generator=g)
    for p in (pg, pe):
        p.reshift(shift)
    for r in rs:
        assert torch.equal(pg.apply(r), pe.apply(r))
        assert torch.equal(pg.apply_transpose(r), pe.apply_transpose(r))


@pytest.mark.parametrize("precision", [32, 64])
def test_dense_coarsest_level_is_solved_exactly(precision):
    """A coarsest level of at most ``dense_max`` unknowns is solved by its dense inverse (the
    reference's coarsest-level inverse): A_c x = b to rounding, and the transpose A_c^T x = b."""
    wl, case, pc, s = _cavity_pc("amg", precision, coarse_solve="auto")
    h = pc.h
    assert h.coarse_solve == "dense" and len(h.levels) >= 2
    pc.refresh(s)
    lv = h.levels[-1]
    g = torch.Generator(device="cuda").manual_seed(2)
    b = torch.randn(lv.n * h.b, dtype=lv.values.dtype, device="cuda", generator=g)
    # fp32: the inverse of an operator of condition ~1e5 leaves a relative residual ~1e-2
    tol = 2e-2 if precision == 32 else 1e-9
    for transpose in (False, True):
        x = h.vcycle(len(h.levels) - 1, b, transpose).clone()
        ax = torch.empty_like(x)
        lv.spmv(x, ax, transpose)
        assert float((ax - b).norm()) <= tol * float(b.norm())
    _, _, pi, _ = _cavity_pc("amg", precision)
    assert pi.h.coarse_solve == "ilu"


@pytest.mark.parametrize("kind", ["ilu", "amg"])
def test_reshift_equals_a_fresh_shifted_preconditioner(kind):
    """The beta-only refresh (new shift, same materialised Jacobian) gives the preconditioner a
    fresh build with that shift gives."""
    wl, case, pc, s = _cavity_pc(kind, 64)
    pc.refresh(s)
    shift = 0.5 + torch.rand(case.n_unknowns, dtype=torch.float64, device="cuda")
    pc.reshift(shift)
    _, _, fresh, _ = _cavity_pc(kind, 64, shift=shift)
    fresh.refresh(s)
    r = torch.randn(case.n_unknowns, dtype=torch.float64, device="cuda")
    assert torch.equal(pc.apply(r), fresh.apply(r))


def test_implicit_adjoint_with_amg_equals_ilu():
    from aquaflux_gb300.amg import AmgPreconditioner
    from aquaflux_gb300.solve import BlockJacobian, implicit_adjoint, newton_solve

    from aquaflux_gb300 import workloads

    wl = workloads.channel3d(10)
    case = wl.device_case()
    res = newton_solve(case, wl.initial_state(), precision=64, max_steps=40, rtol=1e-12)
    assert res.converged
    g = torch.randn(case.n_unknowns, dtype=torch.float64, device="cuda")
    a = implicit_adjoint(case, res.state, g, rtol=1e-12)
    b = implicit_adjoint(case, res.state, g, rtol=1e-12,
                         preconditioner=AmgPreconditioner(BlockJacobian(case), 64, min_cells=100))
    assert a.converged and b.converged
    assert float((a.lam - b.lam).abs().max()) <= 1e-8 * float(a.lam.abs().max())
    assert float((a.dparams - b.dparams).abs().max()) <= 1e-8 * float(a.dparams.abs().max())


def test_batched_jvp_equals_single_jvps():
    from aquaflux_gb300 import workloads

    wl = workloads.channel3d(8)
    case = wl.device_case()
    s = wl.initial_state(noise=0.05)
    vs = torch.randn(3, case.n_unknowns, dtype=torch.float64, device="cuda")
    out = case.jvp_batch(s, vs)
    for i in range(3):
        assert torch.equal(out[i], case.jvp(s, vs[i]))


@pytest.mark.parametrize("precision", [32, 64])
def test_preconditioners_on_one_case_share_its_kept_plan(precision):
    """The second AMG preconditioner on a case reuses the case's connectivity-only plan and level
    structures (FlowCase.pattern_plan, ILU(0) clones) and applies bitwise what the first does, in
    both precisions and through the transpose."""
    from aquaflux_gb300.amg import AmgPreconditioner
    from aquaflux_gb300.solve import BlockJacobian

    wl, case, p1, s = _cavity_pc("amg", precision)
    plans = dict(case._pattern_plans)
    p2 = AmgPreconditioner(BlockJacobian(case), precision, min_cells=150)
    assert case._pattern_plans.keys() == plans.keys()
    kept = [v for k, v in plans.items() if k[0].startswith("amg_hierarchy_structures")]
    assert kept and len(kept[0]["levels"]) == len(p1.h.levels) > 1
    assert p2.h.levels[0].d_indices is p1.h.levels[0].d_indices
    for p in (p1, p2):
        p.refresh(s)
    g = torch.Generator(device="cuda").manual_seed(2)
    r = torch.randn(case.n_unknowns, dtype=torch.float64, device="cuda", generator=g)
    for _ in range(2):  # eager, then the graph replay
        assert torch.equal(p1.apply(r), p2.apply(r))
        assert torch.equal(p1.apply_transpose(r), p2.apply_transpose(r))
