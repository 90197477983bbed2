"""Newton-Krylov on the GPU: Jacobian materialisation, ILU(0) preconditioning, FGMRES, Newton.

Restates, for the GPU, the reference's implicit solve:

* ``ImplicitNewtonSolver`` / ``_forward`` / ``_damped_newton_step`` (``aquaflux/solve/implicit.py:
  458-635, 767-864``): Newton steps to ``||R|| <= atol + rtol ||R_0||`` (``within_tolerance``,
  ``aquaflux/solve/forward_step.py:352``, defaults ``rtol = 1e-10``, ``atol = 1e-12``), each step's
  linear solve inexact (``GMRES(rtol=1e-3, atol=1e-3)``, ``implicit.py:50``), globalised by the
  backtracking line search of ``implicit.py:270-455`` (largest ``alpha`` in ``1, 1/2, ...`` that
  reduces the residual norm, else the shortest rung);
* ``solve_linear`` (``aquaflux/solve/linear.py:199-298``): a right-preconditioned Krylov solve with
  the matrix-free JVP as the operator.  The GMRES itself is a third-party lineax routine in the
  reference; here it is flexible GMRES(m) (right preconditioning, CGS2 orthogonalisation) written
  over torch device tensors, so only converged states -- not Krylov iterates -- are compared;
* the preconditioner: ILU(0) of a materialised block Jacobian (``materialize_block_jacobian``,
  ``aquaflux/solve/sparse_jacobian.py:722-847``) in the cell-major interleaved order
  (``aquaflux/solve/ordering.py:195-242``), factored and applied on the GPU in fp32 (the
  mixed-precision form) or fp64 (the plain form), with the FP64 Newton defect correction outside.
"""
from __future__ import annotations

import dataclasses
import math
import time

import numpy as np
import torch

from ._lib import FvError, check, lib, ptr
from .colouring import block_stencil_colouring, cell_pattern, stencil_pattern
from .ilu0 import Ilu0
from .refresh import StepReport


def _stream() -> int:
    return int(torch.cuda.current_stream().cuda_stream)


class BlockJacobian:
    """The block Jacobian on the reach-``reach`` cell pattern.

    ``frozen=True`` is ``J_direct`` (gradients, SST closure and a_P held fixed), an operator of
    exactly reach 1.  At reach 1 it is assembled directly (``fv_assemble_jacobian``: forward-mode
    face-flux derivatives summed into the block rows, no colouring); ``method="probe"`` recovers
    the same operator by coloured probes of ``fv_jvp_frozen`` as the reference does.
    ``frozen=False`` probes the full JVP (exact when ``reach`` covers the Jacobian's reach, 3 for
    these residuals).  Blocks are cell-major ``b x b`` with ``b`` the number of fields.
    """

    def __init__(self, case, *, reach: int = 1, frozen: bool = True, method: str | None = None,
                 precision: int = 64):
        self.case = case
        if precision not in (32, 64):
            raise ValueError(f"precision must be 64 or 32, got {precision}")
        self.precision = precision  # arithmetic and storage of the direct assembly
        mesh = case.dmesh.mesh
        self.n = mesh.n_cells
        self.b = case.n_unknowns // self.n
        interior = mesh.neighbour >= 0
        self._own, self._nb = mesh.owner[interior], mesh.neighbour[interior]
        self.reach = reach
        def pattern():
            if reach == 1:
                return cell_pattern(self._own, self._nb, self.n)
            pat = stencil_pattern(self._own, self._nb, self.n, reach).tocsr()
            pat.sort_indices()
            return (np.ascontiguousarray(pat.indptr, dtype=np.int32),
                    np.ascontiguousarray(pat.indices, dtype=np.int32))

        plan = getattr(case, "pattern_plan", None)
        self.indptr, self.indices = (plan(("jacobian_pattern", reach), pattern) if plan
                                     else pattern())
        self.nnzb = int(self.indptr[-1])
        self.frozen = frozen
        if method is None:
            method = "assemble" if (frozen and reach == 1) else "probe"
        if method == "assemble" and not (frozen and reach == 1):
            raise ValueError("direct assembly builds the frozen reach-1 Jacobian only")
        if precision == 32 and method != "assemble":
            raise ValueError("the fp32 Jacobian is built by direct assembly only")
        self.method = method
        self._colouring = None
        self.d_indptr = torch.tensor(self.indptr, device="cuda")
        self.d_indices = torch.tensor(self.indices, device="cuda")
        # fp32 assembly stores fp32 blocks (the fp32 preconditioner's own precision)
        self.values = torch.zeros(self.nnzb * self.b * self.b, device="cuda",
                                  dtype=torch.float32 if precision == 32 else torch.float64)

    @property
    def colouring(self):
        if self._colouring is None:
            self._colouring = block_stencil_colouring(self._own, self._nb, self.n, self.reach)
            self.d_colour = torch.tensor(self._colouring.colour.astype(np.int32), device="cuda")
        return self._colouring

    @property
    def n_probes(self) -> int:
        return self.colouring.n_colours * self.b

    def materialize(self, state: torch.Tensor) -> torch.Tensor:
        if self.method == "assemble":
            fn = lib().fv_assemble_jacobian_f32 if self.precision == 32 else \
                lib().fv_assemble_jacobian
            check(fn(self.case.handle, ptr(state), ptr(self.d_indptr), ptr(self.d_indices),
                     ptr(self.values), _stream()))
            return self.values
        n_colours = self.colouring.n_colours
        check(lib().fv_probe_jacobian(self.case.handle, ptr(state), int(self.frozen),
                                      ptr(self.d_colour), n_colours,
                                      ptr(self.d_indptr), ptr(self.d_indices), ptr(self.values),
                                      _stream()))
        return self.values

    def to_scipy(self):
        import scipy.sparse as sp

        v = self.values.cpu().numpy().reshape(-1, self.b, self.b)
        n = self.n * self.b
        return sp.bsr_matrix((v, self.indices, self.indptr), shape=(n, n))


class ShiftedCellMajorOperator:
    """``D (J + diag(shift)) D`` of a :class:`BlockJacobian` on the GPU, pattern fixed.

    ``ShiftedCellMajorOperator.assemble`` (``aquaflux/solve/amg_preconditioner.py:545-658``): the
    pseudo-transient shift (field-major, may be None) on the diagonal, then (``equilibrate``) the
    symmetric square-root-diagonal scale, in the cell-major block layout the Jacobian already has.
    ``assemble`` returns ``(values, scale)``, ``scale`` field-major (None without equilibration);
    the values buffer is reused by the next call.
    """

    def __init__(self, jac: BlockJacobian, *, equilibrate: bool = True, precision: int = 64):
        self.jac = jac
        n, b = jac.n, jac.b
        self.equilibrate = bool(equilibrate)
        self.dtype = torch.float64 if precision == 64 else torch.float32
        self._work = torch.empty(2 * n * b + 1, dtype=torch.float64, device="cuda")
        self.scale = (torch.empty(n * b, dtype=torch.float64, device="cuda")
                      if self.equilibrate else None)
        self.values = torch.empty(jac.nnzb * b * b, dtype=self.dtype, device="cuda")

    def assemble(self, values: torch.Tensor, shift: torch.Tensor | None = None):
        jac = self.jac
        check(lib().fv_bsr_shift_equilibrate(
            jac.n, jac.b, ptr(jac.d_indptr), ptr(jac.d_indices), ptr(values), ptr(shift),
            int(self.equilibrate), ptr(self.scale), ptr(self._work), ptr(self.values),
            int(self.dtype == torch.float64), _stream()))
        return self.values, self.scale


class IluPreconditioner:
    """``M ~= (J + diag(shift))^-1``: ILU(0) of the materialised block Jacobian, fp32 or fp64, on
    the GPU; optionally of the shifted and symmetrically equilibrated operator
    (:class:`ShiftedCellMajorOperator`), ``M = D (D (J + shift) D)_ILU^-1 D``.

    Vectors arrive field-major (the state layout) and are interleaved cell-major (and scaled) for
    the factor by one kernel each way.  ``reshift(shift)`` re-factors for a new shift without
    re-materialising the Jacobian (the beta-only refresh of ``amg_preconditioner.py:909-948``).
    """

    def __init__(self, jac: BlockJacobian, precision: int = 32, *, shift=None,
                 equilibrate: bool = False):
        self.jac = jac
        self.precision = precision
        self.dtype = torch.float32 if precision == 32 else torch.float64
        self.ilu = Ilu0.__new__(Ilu0)
        self.ilu._setup(jac.indptr, jac.indices, jac.b, precision)
        self.shift = None if shift is None else torch.as_tensor(shift, dtype=torch.float64,
                                                                device="cuda")
        self.op = (ShiftedCellMajorOperator(jac, equilibrate=equilibrate, precision=precision)
                   if (shift is not None or equilibrate) else None)
        self._cm = torch.empty(jac.n * jac.b, dtype=self.dtype, device="cuda")
        self._x = torch.empty_like(self._cm)
        self._f64 = int(precision == 64)

    def _factor(self, values):
        if self.op is None:
            self.ilu.refactor(values)
        else:
            vals, _ = self.op.assemble(values, self.shift)
            self.ilu.refactor(vals)

    def refresh(self, state: torch.Tensor) -> None:
        self._factor(self.jac.materialize(state))

    def reshift(self, shift) -> None:
        """New shift on the last materialised Jacobian: re-assemble and re-factor only."""
        if self.op is None:
            self.op = ShiftedCellMajorOperator(self.jac, equilibrate=False,
                                               precision=self.precision)
        self.shift = None if shift is None else torch.as_tensor(shift, dtype=torch.float64,
                                                                device="cuda")
        self._factor(self.jac.values)

    def apply(self, r: torch.Tensor, transpose: bool = False) -> torch.Tensor:
        n, b = self.jac.n, self.jac.b
        scale = None if self.op is None else self.op.scale
        check(lib().fv_to_cells(n, b, 0, ptr(scale), ptr(r), ptr(self._cm), self._f64,
                                _stream()))
        self.ilu.solve(self._cm, transpose=transpose, out=self._x)
        out = torch.empty(n * b, dtype=torch.float64, device="cuda")
        check(lib().fv_from_cells(n, b, 0, ptr(scale), ptr(self._x), self._f64, ptr(out),
                                  _stream()))
        return out

    def apply_transpose(self, r: torch.Tensor) -> torch.Tensor:
        """``M^T r`` (``D`` is diagonal, so only the factor's solve is transposed)."""
        return self.apply(r, transpose=True)


@dataclasses.dataclass
class KrylovResult:
    x: torch.Tensor
    iterations: int
    residual_norm: float
    converged: bool


class KrylovWorkspace:
    """Device storage of FGMRES(m) for vectors of length ``n``, allocated once and reused by every
    solve given it: the Arnoldi basis ``V`` (m + 1, n), the preconditioned basis ``Z`` (m, n), and
    the library's Hessenberg / Givens / reduction workspace (``fv_krylov_create``); plus a pinned
    host buffer the per-iteration residual estimates are copied into."""

    def __init__(self, n: int, m: int):
        import ctypes

        self.n, self.m = int(n), int(m)
        self.V = torch.empty(m + 1, n, dtype=torch.float64, device="cuda")
        self.Z = torch.empty(m, n, dtype=torch.float64, device="cuda")
        self.dnorm = torch.zeros(1, dtype=torch.float64, device="cuda")
        self.est = torch.zeros(m + 1, 2, dtype=torch.float64).pin_memory()
        h = ctypes.c_void_p()
        check(lib().fv_krylov_create(m, ctypes.byref(h)))
        self._h = h

    def norm(self, x: torch.Tensor) -> float:
        """``||x||`` by the workspace's deterministic reduction (waits for the result)."""
        check(lib().fv_krylov_norm(self._h, x.numel(), ptr(x), ptr(self.dnorm), _stream()))
        return float(self.dnorm.item())

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().fv_krylov_destroy(h)
            except Exception:
                pass


def fgmres(matvec, b: torch.Tensor, precond=None, *, rtol: float = 1e-3, atol: float = 0.0,
           restart: int = 30, maxiter: int = 300,
           workspace: KrylovWorkspace | None = None) -> KrylovResult:
    """Flexible GMRES(restart), right-preconditioned, CGS2 orthogonalisation, fp64, on the device.

    The reference's ``solve_linear`` (``aquaflux/solve/linear.py:199-298``) with lineax GMRES.  Each
    Arnoldi step is the library's ``fv_krylov_arnoldi`` (deterministic projections, the Hessenberg
    column, the Givens reduction and the residual estimate ``|g_{j+1}|`` computed on the device);
    the host copies the two-number estimate into pinned memory and reads it only after the next
    iteration has been queued, so the device never waits for the host.  The iteration queued past
    convergence is discarded (its column is not used); near the tolerance, where the estimates'
    decay predicts convergence at the current column, the host reads that column before queueing
    another.  Each cycle ends with ``x += Z y`` (``fv_krylov_update``, the triangular solve on the
    device) and the true residual ``b - A x``.  Results are bitwise identical run to run.
    """
    if not b.is_cuda:
        raise ValueError("fgmres runs on the GPU: b must be a CUDA tensor")
    n = b.numel()
    ws = workspace
    if ws is None or ws.n != n or ws.m < restart:
        ws = KrylovWorkspace(n, restart)
    M = precond if precond is not None else (lambda v: v)
    L = lib()
    x = torch.zeros_like(b)
    bnorm = ws.norm(b)
    tol = max(atol, rtol * bnorm)
    if bnorm <= tol:
        return KrylovResult(x, 0, bnorm, True)
    r, beta, total = b, bnorm, 0
    V, Z, est = ws.V, ws.Z, ws.est
    while total < maxiter:
        m = min(restart, maxiter - total)
        check(L.fv_krylov_start(ws._h, n, ptr(r), ptr(V[0]), 0, _stream()))
        seen = [beta]     # residual estimates read so far in this cycle
        k_done = 0
        pending = None    # (column, event) queued but not yet read

        def read(jp, ev) -> bool:
            """Read column jp's estimate; True when the cycle stops after it."""
            nonlocal k_done, total
            ev.synchronize()
            e, hnext = est[jp].tolist()
            seen.append(e)
            k_done = jp + 1
            total += 1
            return e <= tol or hnext == 0.0

        stop = False
        for j in range(m):
            if pending is not None and len(seen) >= 2:
                # the last estimate read and its decay predict the pending column's estimate
                pred = seen[-1] * min(1.0, seen[-1] / max(seen[-2], 1e-300))
                if pred <= tol:
                    stop = read(*pending)
                    pending = None
                    if stop:
                        break
            Z[j].copy_(M(V[j]))
            w = matvec(Z[j])
            check(L.fv_krylov_arnoldi(ws._h, j, n, ptr(V), ptr(w), ptr(est[j]), _stream()))
            ev = torch.cuda.Event()
            ev.record()
            if pending is not None and read(*pending):
                pending = None
                stop = True
                break
            pending = (j, ev)
        if not stop and pending is not None:
            read(*pending)
        check(L.fv_krylov_update(ws._h, k_done, n, ptr(Z), ptr(x), _stream()))
        r = b - matvec(x)
        beta = ws.norm(r)
        if beta <= tol:
            return KrylovResult(x, total, beta, True)
    return KrylovResult(x, total, beta, False)


@dataclasses.dataclass
class NewtonResult:
    state: torch.Tensor
    converged: bool
    steps: int
    residual_norms: list
    krylov_iterations: list
    seconds: float
    phase_seconds: dict
    refreshes: int = 0  # preconditioner rebuilds (Jacobian materialisations)


def newton_solve(case, state0, *, rtol: float = 1e-10, atol: float = 1e-12, max_steps: int = 50,
                 linear_rtol: float = 1e-3, restart: int = 30,
                 max_krylov: int = 300, precision: int = 32, reach: int = 1, frozen: bool = True,
                 refresh_every: int = 1, line_search_steps: int = 10,
                 preconditioner=None, kind: str = "ilu",
                 precond_options: dict | None = None, tangents: int = 64,
                 refresh_trigger=None, drift_measure=None,
                 linearised: bool | None = None) -> NewtonResult:
    """Newton's method with FGMRES, preconditioned by ILU(0) of the materialised Jacobian
    (``kind="ilu"``) or by an ILU(0)-smoothed aggregation V-cycle (``kind="amg"``), in fp32 or
    fp64 (``precision``).

    ``precision=32`` builds the whole preconditioner in fp32: the frozen Jacobian it is formed
    from is assembled by fp32 dual numbers (``fv_assemble_jacobian_f32``; the values are stored
    in fp32 either way), then factored and applied in fp32.  ``tangents=32`` also evaluates the
    Krylov operator ``J v`` in fp32 arithmetic (``fv_jvp_f32``).  The residual, the Newton
    update, the Krylov orthogonalisation, the line search and the stopping test stay fp64, so the
    root is the fp64 root; only the linear solves, already inexact at ``linear_rtol``, see fp32
    rounding.  The FGMRES bases are allocated once per
    solve (:class:`KrylovWorkspace`).  ``refresh_trigger`` replaces the fixed ``refresh_every``
    schedule: the preconditioner is rebuilt at the first step and then only when the trigger fires
    on the step history since the last rebuild (see :func:`pseudo_transient_solve`).

    ``linearised`` (fp64 tangents): the Krylov operator is the linearised JVP
    (``case.linearise`` at each Newton iterate, the residual evaluations keeping their face
    intermediates, then ``case.jvp_linearised``; the same product within rounding, ``jax.linearize``
    rather than ``jax.jvp``).  ``None`` (default) uses it where the case allows it (first-order
    upwind advection), ``False`` never."""
    if tangents not in (32, 64):
        raise ValueError(f"tangents must be 64 or 32, got {tangents}")
    from ._lib import FvError
    t_all = time.perf_counter()
    s = torch.as_tensor(state0, dtype=torch.float64, device="cuda").clone()
    if preconditioner is None:
        jac = BlockJacobian(case, reach=reach, frozen=frozen,
                            precision=32 if (precision == 32 and frozen and reach == 1) else 64)
        if kind == "amg":
            from .amg import AmgPreconditioner

            preconditioner = AmgPreconditioner(jac, precision, **(precond_options or {}))
        else:
            preconditioner = IluPreconditioner(jac, precision)
    kws = KrylovWorkspace(s.numel(), restart)
    torch.cuda.synchronize()
    # "setup": pattern, hierarchy plan and factor structures (host work, once per solve here);
    # "precond_setup": the per-refresh materialisation and factorisation
    phases = {"setup": time.perf_counter() - t_all, "residual": 0.0, "precond_setup": 0.0,
              "krylov": 0.0, "line_search": 0.0}

    def timed(key, fn, *a):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn(*a)
        torch.cuda.synchronize()
        phases[key] += time.perf_counter() - t0
        return out

    lin = tangents == 64 and linearised is not False
    lin_point = None  # the iterate whose evaluation the case holds for the linearised JVP
    if lin:
        try:
            r = timed("residual", case.linearise, s)
            lin_point = s
        except FvError:
            if linearised:
                raise
            lin = False
    if not lin:
        r = timed("residual", case.residual, s)
    evaluate = case.linearise if lin else case.residual
    norms = [kws.norm(r)]
    target = atol + rtol * norms[0]
    its = []
    converged = norms[0] <= target
    step = 0
    history, drift_fn, refreshes = [], None, 0
    while not converged and step < max_steps:
        if (refresh_trigger.should_refresh(history) or refreshes == 0
                if refresh_trigger is not None else step % refresh_every == 0):
            timed("precond_setup", preconditioner.refresh, s)
            refreshes += 1
            history = []
            drift_fn = drift_measure(s) if drift_measure is not None else None
        if lin and lin_point is not s:  # the accepted iterate was not the last one evaluated
            r = timed("residual", case.linearise, s)
            lin_point = s
        matvec = ((lambda v: case.jvp_linearised(s, v)) if lin else
                  (lambda v: case.jvp(s, v, precision=tangents)))
        res = timed("krylov", lambda: fgmres(matvec, -r, preconditioner.apply,
                                             rtol=linear_rtol, restart=restart,
                                             maxiter=max_krylov, workspace=kws))
        its.append(res.iterations)
        delta = res.x

        def search():
            nonlocal lin_point
            ref = norms[-1]
            best = None
            alpha = 1.0
            for _ in range(line_search_steps + 1):
                cand = s + alpha * delta
                rc = evaluate(cand)
                lin_point = cand
                nc = kws.norm(rc)
                if math.isfinite(nc):
                    best = (cand, rc, nc) if best is None or nc < best[2] else best
                    if nc < ref:
                        return cand, rc, nc
                alpha *= 0.5
            if best is not None:
                return best
            cand = s + alpha * delta
            lin_point = cand
            return cand, evaluate(cand), float("nan")

        s, r, nrm = timed("line_search", search)
        norms.append(nrm)
        step += 1
        converged = nrm <= target
        if not math.isfinite(nrm):
            break
        history.append(StepReport(len(history), int(res.iterations), nrm, nrm / norms[0],
                                  drift_fn(s) if drift_fn is not None else 0.0))
    torch.cuda.synchronize()
    return NewtonResult(s, converged, step, norms, its, time.perf_counter() - t_all, phases,
                        refreshes)


def reynolds_scales(n_points: int, ratio: float = 10.0) -> tuple[float, ...]:
    """The molecular-viscosity factors of a Reynolds continuation, ``(ratio ** N, ..., ratio,
    1.0)`` for ``N = n_points`` (``GeometricReynoldsSchedule.scales``,
    ``aquaflux/turbulence/reynolds.py:96-132``): one decade of Reynolds number per point by
    default, ending at the target."""
    if n_points < 0:
        raise ValueError(f"n_points must be >= 0, got {n_points}")
    return tuple(float(ratio ** (n_points - i)) for i in range(n_points + 1))


@dataclasses.dataclass
class ReynoldsContinuationResult:
    state: torch.Tensor      # the target-Reynolds root
    converged: bool          # the target solve's convergence
    points: list             # per point: viscosity scale, Newton steps, Krylov iterations, seconds
    seconds: float


def reynolds_continuation(case, state0, n_points: int, *, ratio: float = 10.0,
                          intermediate_rtol: float | None = 1e-2,
                          intermediate_atol: float | None = None,
                          **newton_kwargs) -> ReynoldsContinuationResult:
    """Newton's method by Reynolds-number continuation (``solve_reynolds_continuation``,
    ``aquaflux/turbulence/reynolds.py:144-338``): ``n_points`` lower-Reynolds solves, the case's
    molecular viscosity scaled by :func:`reynolds_scales`, each seeded by the previous converged
    state and converged loosely (``intermediate_rtol`` / ``intermediate_atol`` replace ``rtol`` /
    ``atol`` there), then the solve at the case's own viscosity with the caller's tolerances.  The
    path changes, the root does not.  A lower point that fails raises ``RuntimeError`` naming it;
    the case's viscosity is restored in every outcome."""
    scales = reynolds_scales(n_points, ratio)
    mu0 = case.mu
    t0 = time.perf_counter()
    seed = state0
    points = []
    ramp = dict(newton_kwargs)
    if intermediate_rtol is not None:
        ramp["rtol"] = intermediate_rtol
    if intermediate_atol is not None:
        ramp["atol"] = intermediate_atol
    try:
        for i, scale in enumerate(scales[:-1]):
            case.set_params(mu=mu0 * scale)
            res = newton_solve(case, seed, **ramp)
            points.append({"viscosity_scale": scale, "converged": bool(res.converged),
                           "newton_steps": res.steps,
                           "krylov_iterations": int(sum(res.krylov_iterations)),
                           "seconds": round(res.seconds, 3)})
            if not res.converged:
                raise RuntimeError(
                    f"Reynolds-continuation point {i + 1} of {n_points} (molecular viscosity "
                    f"scaled by {scale:g}, i.e. Reynolds number reduced by {scale:g}x) failed to "
                    f"converge. Increase n_points for a gentler ramp, or check the case at this "
                    f"Reynolds number directly.")
            seed = res.state
    finally:
        case.set_params(mu=mu0)
    res = newton_solve(case, seed, **newton_kwargs)
    points.append({"viscosity_scale": 1.0, "converged": bool(res.converged),
                   "newton_steps": res.steps, "krylov_iterations": int(sum(res.krylov_iterations)),
                   "seconds": round(res.seconds, 3)})
    return ReynoldsContinuationResult(res.state, bool(res.converged), points,
                                      time.perf_counter() - t0)


class TransposedPreconditioner:
    """``M^T`` of a preconditioner with an exact transposed application (``apply_transpose``: the
    transposed ILU(0) solve, or the transposed V-cycle), as the reference's
    ``TransposedPreconditioner`` / ``jax.linear_transpose`` (``aquaflux/solve/implicit.py:709-730``)."""

    def __init__(self, pc):
        self.pc = pc

    def apply(self, r: torch.Tensor) -> torch.Tensor:
        return self.pc.apply_transpose(r)


@dataclasses.dataclass
class AdjointResult:
    lam: torch.Tensor           # adjoint state: J^T lam = g
    dparams: torch.Tensor       # (d/dmu, d/d inlet_scale) of the objective
    krylov_iterations: int
    converged: bool


def implicit_adjoint(case, state, g, *, rtol: float = 1e-10, precision: int = 64,
                     restart: int = 30, max_krylov: int = 1000,
                     preconditioner=None) -> AdjointResult:
    """Implicit-function-theorem gradient at a converged root (``_implicit_solve_bwd``,
    ``aquaflux/solve/implicit.py:733-761``): solve ``J^T lam = g`` with FGMRES on the hand-written
    VJP (its forward pass held once, ``case.hold_forward``) and the transposed ILU(0) preconditioner (the reference's tight 1e-10 adjoint solve,
    ``aquaflux/solve/linear.py:40-42``), then ``dL/dtheta = -lam^T dR/dtheta`` for
    ``theta = (mu, inlet_scale)``.  ``preconditioner``: any with ``refresh`` and
    ``apply_transpose`` (ILU(0) by default; the AMG V-cycle has an exact transpose too)."""
    s = torch.as_tensor(state, dtype=torch.float64, device="cuda")
    gv = torch.as_tensor(g, dtype=torch.float64, device="cuda")
    if preconditioner is None:
        preconditioner = IluPreconditioner(BlockJacobian(case, reach=1, frozen=True), precision)
    preconditioner.refresh(s)
    mt = TransposedPreconditioner(preconditioner)
    # the forward pass held once (the preconditioner's refresh above is the last other evaluation):
    # every Krylov product then runs the adjoint stages only
    case.hold_forward(s)

    def adjoint_product(w):
        try:
            return case.vjp_held(s, w)
        except FvError as e:
            if "no forward pass held" not in str(e):
                raise
            # a preconditioner that evaluates the case dropped the hold: hold it again
            case.hold_forward(s)
            return case.vjp_held(s, w)

    res = fgmres(adjoint_product, gv, mt.apply, rtol=rtol, restart=restart, maxiter=max_krylov)
    dparams = -case.param_vjp(s, res.x)
    return AdjointResult(res.x, dparams, res.iterations, res.converged)


@dataclasses.dataclass
class FunctionalGradient:
    value: float
    dparams: torch.Tensor   # total dJ/d(mu, inlet_scale)
    dnodes: torch.Tensor | None  # total dJ/dnodes, (n_nodes, dim)
    adjoint: AdjointResult


def functional_gradient(case, state, weights, *, viscous_only: bool = False, nodes: bool = True,
                        rtol: float = 1e-10, preconditioner=None) -> FunctionalGradient:
    """Total derivative of a face-flux functional ``J(state(theta), theta)`` at a converged state
    by the implicit function theorem (``_implicit_solve_bwd``, ``aquaflux/solve/implicit.py:
    733-761``): ``J^T lam = dJ/dstate``, then ``dJ/dtheta = dJ/dtheta|_state - lam^T dR/dtheta``
    for ``theta`` = (mu, inlet_scale) and every node coordinate."""
    f = case.face_functional(state, weights, viscous_only=viscous_only, nodes=nodes)
    adj = implicit_adjoint(case, state, f["dstate"], rtol=rtol, preconditioner=preconditioner)
    dparams = f["dparams"] + adj.dparams
    dnodes = None
    if nodes:
        dnodes = f["dnodes"] - case.node_vjp(state, adj.lam)
    return FunctionalGradient(f["value"], dparams, dnodes, adj)


@dataclasses.dataclass
class BatchedGradients:
    value: torch.Tensor      # (n_instances,) objective of each instance
    dmu: torch.Tensor        # (n_instances,) dJ_i / dmu_i
    dvelocity: torch.Tensor  # (n_instances,) dJ_i / dU_i
    adjoint: AdjointResult


def batched_gradients(case, state, bw, *, rtol: float = 1e-10,
                      preconditioner=None) -> BatchedGradients:
    """Per-instance gradients of the batched calibration sweep (independent instances side by side
    in one disjoint-union case): the objective of instance ``i`` is ``g . state`` over its cells
    (its mean outlet velocity); one adjoint solve ``J^T lam = g`` serves every instance (``J`` is
    block diagonal), and ``dJ_i/dtheta_i = -lam_i . dR/dtheta`` with the viscosity / inlet tangents
    seeded on every instance at once, reduced per instance (``fv_segment_dot``)."""
    areas = case.dmesh.geometry()["area"].cpu().numpy()
    g = torch.tensor(bw.outlet_weights(areas), device="cuda")
    s = torch.as_tensor(state, dtype=torch.float64, device="cuda")
    seg = torch.tensor(bw.offsets, dtype=torch.int32, device="cuda")
    nfld = case.n_unknowns // case.n_cells
    n = bw.n_instances

    def seg_dot(a, b):
        out = torch.empty(n, dtype=torch.float64, device="cuda")
        check(lib().fv_segment_dot(n, ptr(seg), nfld, case.n_cells, ptr(a), ptr(b), ptr(out),
                                   _stream()))
        return out

    value = seg_dot(g, s)
    adj = implicit_adjoint(case, s, g, rtol=rtol, preconditioner=preconditioner)
    dmu_vec, dsc_vec = case.param_jvp(s)
    dmu = -seg_dot(adj.lam, dmu_vec)
    dvel = -seg_dot(adj.lam, dsc_vec) / torch.tensor(bw.velocity, device="cuda")
    return BatchedGradients(value, dmu, dvel, adj)


@dataclasses.dataclass
class ContinuationResult:
    state: torch.Tensor
    converged: bool
    steps: int
    residual_norms: list
    betas: list
    escalations: int
    krylov_iterations: list
    seconds: float
    refreshes: int = 0  # Jacobian materialisations (the rest of the steps re-shifted only)


def shift_basis(jac: BlockJacobian, velocity_only: bool = False,
                fixed_rows: torch.Tensor | None = None) -> torch.Tensor:
    """The base pseudo-time shift ``d`` (field-major): the magnitude of the frozen Jacobian's
    diagonal on the momentum rows (the momentum diagonal ``a_P``, ``LocalCourantBasis`` with weight
    1, ``aquaflux/solve/shift_basis.py:62-91``) and, unless ``velocity_only``, on the k / omega rows;
    zero on the continuity rows (``MomentumShiftPolicy``, ``aquaflux/flow/continuation.py:111-186``).
    Uses the values the Jacobian last materialised."""
    n, b = jac.n, jac.b
    if not hasattr(jac, "_diag_blocks"):
        rows = np.repeat(np.arange(n), np.diff(jac.indptr))
        jac._diag_blocks = torch.tensor(np.flatnonzero(rows == jac.indices), device="cuda")
    blocks = jac.values.view(-1, b, b)[jac._diag_blocks]  # (n, b, b)
    d = torch.diagonal(blocks, dim1=1, dim2=2).abs().t().contiguous()  # (b, n)
    dim = b - 1 if b in (3, 4) else b - 3
    d[dim] = 0.0  # continuity
    if velocity_only:
        d[dim + 1:] = 0.0
    d = d.reshape(-1)
    if fixed_rows is not None:  # algebraic rows (the near-wall omega fixation) take no shift
        d[fixed_rows] = 0.0
    return d


def jacobian_diagonal(jac: BlockJacobian) -> torch.Tensor:
    """The scalar diagonal of the last materialised Jacobian, field-major ``(b * n,)``."""
    n, b = jac.n, jac.b
    if not hasattr(jac, "_diag_blocks"):
        rows = np.repeat(np.arange(n), np.diff(jac.indptr))
        jac._diag_blocks = torch.tensor(np.flatnonzero(rows == jac.indices), device="cuda")
    blocks = jac.values.view(-1, b, b)[jac._diag_blocks]
    return torch.diagonal(blocks, dim1=1, dim2=2).t().reshape(-1)


class RowScaledMeasure:
    """The row-equilibrated, field-normalised progress measure of a coupled residual
    (``RowScaledNorm`` / ``coupled_scaled_norm``, ``aquaflux/solve/norm.py:90-200``,
    ``aquaflux/turbulence/coupled.py:1073-1168``), frozen at one state:
    ``m(R) = || [ mean_c(|R_bc| / a_bc) / s_b ]_b ||_2`` over the field blocks ``b``.

    Row scales ``a``: the row's own diagonal of the (solved-variable) Jacobian, so a near-wall
    omega row written as a log ratio passes through with its unit derivative.  Field scales ``s``:
    ``mean|u|`` for the velocity blocks, ``mean(phi / (dphi/dw))`` for k and omega (``mean|phi|``
    when solved directly, exactly 1 for a log-solved field).  Continuity differs from the
    reference, which divides the mass imbalance by the cell's mass throughput: here the row is
    divided by its pressure diagonal and the block by the mean dynamic-plus-static pressure
    magnitude ``mean|p| + rho mean|u|^2 / 2``, making it a fractional pressure change."""

    def __init__(self, case, jac: BlockJacobian, state: torch.Tensor):
        n, b, d = jac.n, jac.b, case.dim
        tiny = 1e-300
        self.n, self.b = n, b
        self.row = jacobian_diagonal(jac).abs() + tiny
        phys = case.to_physical(state) if case.turbulent else state
        u = phys[: d * n]
        umean = float(u.abs().mean())
        p = phys[d * n:(d + 1) * n]
        scales = [umean] * d + [float(p.abs().mean()) + 0.5 * case.rho * umean ** 2]
        if case.turbulent:
            for i, tr in enumerate((case.k_transform, case.omega_transform)):
                blk = phys[(d + 1 + i) * n:(d + 2 + i) * n]
                scales.append(1.0 if tr == "log" else float(blk.abs().mean()))
        self.field = torch.tensor([max(x, tiny) for x in scales], dtype=torch.float64,
                                  device="cuda")

    def per_block(self, r: torch.Tensor) -> torch.Tensor:
        return (r.abs() / self.row).view(self.b, self.n).mean(dim=1) / self.field

    def __call__(self, r: torch.Tensor) -> float:
        return float(torch.linalg.vector_norm(self.per_block(r)))


def positive_projection(state: torch.Tensor, delta: torch.Tensor, start: int, stop: int,
                        tau: float = 0.99, floor: float = 0.0) -> torch.Tensor:
    """Clip each entry's own correction so ``state[start:stop]`` stays positive:
    ``delta_i <- max(delta_i, -tau (phi_i + floor))`` (``positive_block_projection``,
    ``aquaflux/solve/implicit.py:197-300``).  Inactive at a root (``delta = 0``)."""
    out = delta.clone()
    out[start:stop] = torch.maximum(delta[start:stop], -tau * (state[start:stop] + floor))
    return out


def pseudo_transient_solve(case, state0, *, beta0: float = 2.0, exponent: float = 1.0,
                           beta_floor: float = 0.0, max_escalations: int = 6,
                           escalation_factor: float = 2.0, divergence_cap: float = 10.0,
                           rtol: float = 1e-10, atol: float = 1e-12, max_steps: int = 200,
                           linear_rtol: float = 1e-3, restart: int = 30, max_krylov: int = 300,
                           kind: str = "amg", precision: int = 32,
                           velocity_only: bool = False, measure: str = "euclidean",
                           scaled_tol: float | None = None, k_positive: bool = False,
                           k_floor: float = 0.0, backtrack: int = 0,
                           refresh_trigger=None, drift_measure=None,
                           log=None) -> ContinuationResult:
    """Pseudo-transient continuation (``PseudoTransientStep``, ``aquaflux/solve/continuation.py:
    333-735``): each step solves ``(J + beta d) delta = -R`` (the true JVP plus the shift,
    ``fv_jvp_shift``; right-preconditioned FGMRES with the preconditioner built at the same shifted
    diagonal), with the switched-evolution-relaxation schedule ``beta = max(beta_floor,
    beta0 (||R|| / ||R0||)^exponent)`` (``relaxation.py:53-95``) and the divergence guard: a
    candidate is accepted unless it is non-finite or ``||R|| > divergence_cap ||R0||``; otherwise
    ``beta`` grows by ``escalation_factor`` and the step is re-solved (re-factoring the
    preconditioner at the new shift without re-materialising the Jacobian), up to
    ``max_escalations`` times.  ``beta -> 0`` at the root recovers Newton's step.

    ``measure="row_scaled"`` steers the schedule and the guard by :class:`RowScaledMeasure`
    (rebuilt at every outer step from the Jacobian materialised there, held fixed across its
    escalations), and stops when that measure falls to ``scaled_tol`` (or the Euclidean test
    passes).  ``k_positive`` clips each k correction of a directly-solved k so k stays positive
    (:func:`positive_projection` with ``k_floor``).  ``backtrack`` > 0 first halves a rejected step
    up to that many times (a backtracking line search along the shifted Newton direction, as
    ``backtracking_line_search`` does for the plain Newton step) before the shift escalates: on
    a saddle-point system a larger momentum shift leaves continuity to the pressure alone and can
    lengthen the step rather than damp it.  ``log`` receives one dict per attempt.

    ``refresh_trigger`` (a :mod:`aquaflux_gb300.refresh` trigger): the Jacobian is materialised at
    the first step and again only when the trigger fires on the segment's step history; the steps
    in between re-form the preconditioner at their own shift from the frozen Jacobian (the
    beta-only refresh, ``amg_preconditioner.py:909-948``).  Without one the Jacobian is
    re-materialised at every step.  ``drift_measure``: ``reference_state -> (state -> drift)``
    (e.g. :func:`aquaflux_gb300.refresh.eddy_viscosity_drift`), re-based at every refresh."""
    from .amg import AmgPreconditioner

    t_all = time.perf_counter()
    s = torch.as_tensor(state0, dtype=torch.float64, device="cuda").clone()
    jac = BlockJacobian(case)
    zero = torch.zeros(case.n_unknowns, dtype=torch.float64, device="cuda")
    if kind == "amg":
        pc = AmgPreconditioner(jac, precision, shift=zero)
    else:
        pc = IluPreconditioner(jac, precision, shift=zero)
    r = case.residual(s)
    norms = [float(torch.linalg.vector_norm(r))]
    r0 = norms[0]
    target = atol + rtol * r0
    scaled = measure == "row_scaled"
    if measure not in ("euclidean", "row_scaled"):
        raise ValueError(f"measure must be 'euclidean' or 'row_scaled', got {measure!r}")
    kpos = k_positive and case.turbulent and case.k_transform == "direct"
    n, dim = case.n_cells, case.dim
    fixed = None
    if case.turbulent:  # the near-wall omega rows (FixedValueCells) are not shifted
        fixed = torch.as_tensor((dim + 2) * n + case.wall_cells, device="cuda")
    betas, its = [], []
    escalations = 0
    step = 0
    converged = norms[0] <= target
    m0 = m_cur = None
    history, drift_fn, refreshes = [], None, 0
    while not converged and step < max_steps:
        if refresh_trigger is None or refreshes == 0 or refresh_trigger.should_refresh(history):
            pc.shift = zero
            pc.refresh(s)  # materialise J at s (its diagonal also gives the shift basis)
            refreshes += 1
            history = []
            drift_fn = drift_measure(s) if drift_measure is not None else None
        if scaled:
            meas = RowScaledMeasure(case, jac, s)
            m_cur = meas(r)
            if m0 is None:
                m0 = m_cur
            ratio, cap_ref = m_cur / m0, m0
        else:
            meas = None
            ratio, cap_ref = norms[-1] / r0, r0
        if scaled and scaled_tol is not None and m_cur <= scaled_tol:
            converged = True
            break
        beta = max(beta_floor, beta0 * ratio ** exponent)
        d = shift_basis(jac, velocity_only, fixed)
        accepted = False
        for attempt in range(max_escalations + 1):
            shift = beta * d
            pc.reshift(shift)
            res = fgmres(lambda v: case.jvp_shift(s, v, shift), -r, pc.apply, rtol=linear_rtol,
                         restart=restart, maxiter=max_krylov)
            dx = res.x
            if kpos:
                dx = positive_projection(s, dx, (dim + 1) * n, (dim + 2) * n, floor=k_floor)
            its.append(res.iterations)
            alpha = 1.0
            for _ in range(backtrack + 1):
                cand = s + alpha * dx
                rc = case.residual(cand)
                nc = float(torch.linalg.vector_norm(rc))
                mc = meas(rc) if scaled else nc
                ok = math.isfinite(nc) and math.isfinite(mc) and mc <= divergence_cap * cap_ref
                if backtrack:  # a line search asks for decrease, not only for no divergence
                    ok = ok and mc < (m_cur if scaled else norms[-1])
                if ok:
                    break
                alpha *= 0.5
            if log is not None:
                log({"step": step, "attempt": attempt, "beta": beta, "alpha": alpha, "norm": nc,
                     "measure": mc if scaled else None, "accepted": ok,
                     "krylov": res.iterations, "krylov_converged": res.converged,
                     "blocks": meas.per_block(rc).tolist() if scaled else None})
            if ok:
                accepted = True
                break
            beta *= escalation_factor
            escalations += 1
        if not accepted:
            break
        s, r = cand, rc
        norms.append(nc)
        betas.append(beta)
        step += 1
        converged = nc <= target
        history.append(StepReport(len(history), int(res.iterations), nc, nc / r0,
                                  drift_fn(s) if drift_fn is not None else 0.0))
    torch.cuda.synchronize()
    return ContinuationResult(s, converged, step, norms, betas, escalations, its,
                              time.perf_counter() - t_all, refreshes)
