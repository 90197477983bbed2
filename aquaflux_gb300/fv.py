"""Device handles over the C ABI: :class:`DeviceMesh` and :class:`FlowCase`.

These own the library objects (``FvMesh``, ``FvCase``) and pass torch CUDA tensors to the kernels
on torch's current stream.  Every call goes to ``libfvgb.so``; there is no CPU path.

Boundary conditions are given per named patch, as in the reference's ``BoundaryConditions``
(``aquaflux/boundary/collection.py:72-137``):

* ``flow_bc``: ``{patch: ("wall",) | ("moving", U) | ("inlet", U) | ("outlet", p)}`` -- the
  ``NoSlipWall`` / ``MovingWall`` / ``VelocityInlet`` / ``PressureOutlet`` closures of
  ``aquaflux/flow/boundary.py:278-446``;
* ``sst``: ``None`` or ``{"walls": [patches], "k": {patch: ("dirichlet", v) | ("zerograd",)},
  "omega": {...}}`` -- ``SSTTurbulence.build``'s wall patches and scalar closures
  (``aquaflux/turbulence/transport.py:198-243``).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from ._lib import FvCaseDesc, check, lib, ptr
from .mesh import MeshData

FLOW_KIND = {"wall": 0, "moving": 1, "inlet": 2, "outlet": 3}


def _stream() -> int:
    return int(torch.cuda.current_stream().cuda_stream)


class DeviceMesh:
    """A mesh resident on the GPU with its geometry (``Mesh`` + ``Mesh.geometry()``)."""

    def __init__(self, mesh: MeshData):
        mesh.validate()
        self.mesh = mesh
        self.dim, self.n_cells, self.n_faces = mesh.dim, mesh.n_cells, mesh.n_faces
        h = ctypes.c_void_p()
        nodes = np.ascontiguousarray(mesh.nodes, dtype=np.float64)
        off = np.ascontiguousarray(mesh.fn_offsets, dtype=np.int32)
        idx = np.ascontiguousarray(mesh.fn_indices, dtype=np.int32)
        own = np.ascontiguousarray(mesh.owner, dtype=np.int32)
        nb = np.ascontiguousarray(mesh.neighbour, dtype=np.int32)
        check(lib().fv_mesh_create(mesh.dim, mesh.n_cells, mesh.n_faces, mesh.n_nodes, ptr(nodes),
                                   ptr(off), ptr(idx), ptr(own), ptr(nb), _stream(),
                                   ctypes.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def geometry(self) -> dict:
        """Face area / normal / centroid and cell volume / centroid (reference face order)."""
        dev = torch.device("cuda")
        F, C, D = self.n_faces, self.n_cells, self.dim
        out = {"area": torch.empty(F, dtype=torch.float64, device=dev),
               "normal": torch.empty(F, D, dtype=torch.float64, device=dev),
               "face_centroid": torch.empty(F, D, dtype=torch.float64, device=dev),
               "volume": torch.empty(C, dtype=torch.float64, device=dev),
               "cell_centroid": torch.empty(C, D, dtype=torch.float64, device=dev)}
        check(lib().fv_mesh_geometry(self._h, ptr(out["area"]), ptr(out["normal"]),
                                     ptr(out["face_centroid"]), ptr(out["volume"]),
                                     ptr(out["cell_centroid"]), _stream()))
        return out

    def set_nodes(self, nodes: torch.Tensor) -> None:
        nodes = nodes.to(device="cuda", dtype=torch.float64).contiguous()
        check(lib().fv_mesh_set_nodes(self._h, ptr(nodes), _stream()))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().fv_mesh_destroy(h)
            except Exception:
                pass


def case_tables(mesh: MeshData, flow_bc: dict, sst: dict | None):
    """Per-face boundary tables (reference face order) for ``fv_case_create``."""
    F, D = mesh.n_faces, mesh.dim
    kind = np.full(F, -1, dtype=np.int8)
    vel = np.zeros((F, D))
    pb = np.zeros(F)
    for name, spec in flow_bc.items():
        faces = np.asarray(mesh.patches[name], dtype=np.int64)
        if np.any(mesh.neighbour[faces] >= 0):
            raise ValueError(f"patch {name!r} contains interior faces")
        kind[faces] = FLOW_KIND[spec[0]]
        if spec[0] in ("moving", "inlet"):
            vel[faces] = np.asarray(spec[1], dtype=float)
        elif spec[0] == "outlet":
            pb[faces] = float(spec[1])
    t = {"flow_kind": kind, "flow_vel": vel, "flow_p": pb}
    if sst is not None:
        for fld in ("k", "omega"):
            kk = np.full(F, -1, dtype=np.int8)
            vv = np.zeros(F)
            for name, spec in sst[fld].items():
                faces = np.asarray(mesh.patches[name], dtype=np.int64)
                kk[faces] = 0 if spec[0] == "dirichlet" else 1
                if spec[0] == "dirichlet":
                    vv[faces] = float(spec[1])
            t[fld + "_kind"], t[fld + "_val"] = kk, vv
        wall = np.zeros(F, dtype=np.uint8)
        for name in sst["walls"]:
            wall[np.asarray(mesh.patches[name], dtype=np.int64)] = 1
        t["sst_wall"] = wall
    return t


class FlowCase:
    """``MomentumContinuity`` (laminar) or ``CoupledRANS`` (k-omega SST) on the GPU.

    First-order upwind advection (``advection=None``) or limited linear upwind
    (``advection={"k": K}``: ``LimitedUpwind(VenkatakrishnanLimiter(k=K))``, ``K`` None for the
    unlimited reconstruction); compact Green-Gauss gradients (``gradient=None``) or corrected
    Green-Gauss by ``SweptGradientSolve`` (``gradient={"sweeps": s, "relaxation": r}``,
    ``aquaflux/schemes/gradient.py:547-705, 1122-1337``); constant viscosity ``mu`` and density
    ``rho``; optional pressure pin (``FixedValueCells`` on the continuity row).
    """

    def __init__(self, dmesh: DeviceMesh, *, mu: float, rho: float, flow_bc: dict,
                 pressure_pin: int | None = None, pressure_pin_value: float = 0.0,
                 sst: dict | None = None, gradient: dict | None = None,
                 advection: dict | None = None, k_transform: str = "direct",
                 omega_transform: str = "direct", scalar_advection=None):
        self.dmesh = dmesh
        mesh = dmesh.mesh
        self.dim, self.n_cells = mesh.dim, mesh.n_cells
        self.turbulent = sst is not None
        t = case_tables(mesh, flow_bc, sst)
        # SST wall cells: owners of the SST wall faces, whose omega rows are the fixation
        self.wall_cells = (np.unique(mesh.owner[t["sst_wall"] != 0]).astype(np.int64)
                           if sst is not None else np.zeros(0, dtype=np.int64))
        mu_arr = np.asarray(mu, dtype=np.float64)
        mu_field = None
        if mu_arr.ndim == 1:  # a per-cell viscosity field (laminar instances side by side)
            if mu_arr.shape != (mesh.n_cells,):
                raise ValueError(f"a viscosity field needs {mesh.n_cells} values")
            mu_field = mu_arr
            mu_const = float(mu_arr.mean())
        else:
            mu_const = float(mu_arr)
        adv_kind, adv_k = 0, 0.0
        if advection is not None:
            adv_kind = 1 if advection.get("k") is None else 2
            adv_k = 0.0 if advection.get("k") is None else float(advection["k"])
        self.advection = advection
        sweeps = 0 if gradient is None else int(gradient["sweeps"])
        relax = 1.0 if gradient is None else float(gradient.get("relaxation", 1.0))
        self.gradient = gradient
        for name, tr in (("k_transform", k_transform), ("omega_transform", omega_transform)):
            if tr not in ("direct", "log"):
                raise ValueError(f"{name} must be 'direct' or 'log', got {tr!r}")
        self.k_transform, self.omega_transform = k_transform, omega_transform
        transform = (k_transform == "log") | ((omega_transform == "log") << 1)
        if transform and sst is None:
            raise ValueError("the log transforms apply to the k and omega of a turbulent case")
        # k / omega advection: None = the momentum scheme, "upwind", or a dict like `advection`
        s_kind, s_k = 0, 0.0
        if scalar_advection is not None:
            if sst is None:
                raise ValueError("scalar_advection applies to the k and omega of a turbulent case")
            if scalar_advection == "upwind":
                s_kind = 1
            else:
                s_kind = 2 if scalar_advection.get("k") is None else 3
                s_k = 0.0 if scalar_advection.get("k") is None else float(scalar_advection["k"])
        self.scalar_advection = scalar_advection
        desc = FvCaseDesc(1 if sst is not None else 0, mu_const, float(rho),
                          -1 if pressure_pin is None else int(pressure_pin),
                          float(pressure_pin_value), sweeps, relax, adv_kind, adv_k, transform,
                          s_kind, s_k)
        h = ctypes.c_void_p()
        arrs = [np.ascontiguousarray(t.get(k)) if t.get(k) is not None else None
                for k in ("flow_kind", "flow_vel", "flow_p", "k_kind", "k_val", "omega_kind",
                          "omega_val", "sst_wall")]
        check(lib().fv_case_create(dmesh.handle, ctypes.byref(desc), *[ptr(a) for a in arrs],
                                   _stream(), ctypes.byref(h)))
        self._h = h
        self._keep = arrs
        self.n_unknowns = int(lib().fv_case_n_unknowns(h))
        self.mu, self.rho, self.inlet_scale = float(mu_const), float(rho), 1.0
        self.mu_field = None
        if mu_field is not None:
            self.mu_field = torch.as_tensor(mu_field, dtype=torch.float64, device="cuda")
            check(lib().fv_case_set_viscosity_field(h, ptr(self.mu_field), _stream()))

    @property
    def handle(self):
        return self._h

    def set_params(self, mu: float | None = None, inlet_scale: float | None = None) -> None:
        if mu is not None:
            self.mu = float(mu)
        if inlet_scale is not None:
            self.inlet_scale = float(inlet_scale)
        check(lib().fv_case_set_params(self._h, self.mu, self.inlet_scale))

    def _log_blocks(self):
        n, d = self.n_cells, self.dim
        return [slice((d + 1 + i) * n, (d + 2 + i) * n)
                for i, tr in enumerate((self.k_transform, self.omega_transform)) if tr == "log"]

    def to_solved(self, state):
        """Physical ``[u.., p, k, omega]`` -> the solved variables of this case (``log`` on the
        log-transformed blocks, ``CoupledRANS.solved_state``,
        ``aquaflux/turbulence/coupled.py:383-392``)."""
        out = state.clone() if torch.is_tensor(state) else np.array(state, dtype=np.float64)
        for sl in self._log_blocks():
            out[sl] = torch.log(out[sl]) if torch.is_tensor(out) else np.log(out[sl])
        return out

    def to_physical(self, state):
        """Solved variables -> physical ``[u.., p, k, omega]`` (``exp`` on the log blocks,
        ``CoupledRANS.physical_fields``, ``coupled.py:366-381``)."""
        out = state.clone() if torch.is_tensor(state) else np.array(state, dtype=np.float64)
        for sl in self._log_blocks():
            out[sl] = torch.exp(out[sl]) if torch.is_tensor(out) else np.exp(out[sl])
        return out

    def _vec(self, x) -> torch.Tensor:
        x = torch.as_tensor(x, dtype=torch.float64, device="cuda").contiguous()
        if x.shape != (self.n_unknowns,):
            raise ValueError(f"expected a state of shape ({self.n_unknowns},), got {tuple(x.shape)}")
        return x

    def residual(self, state, out: torch.Tensor | None = None) -> torch.Tensor:
        s = self._vec(state)
        r = torch.empty_like(s) if out is None else out
        check(lib().fv_residual(self._h, ptr(s), ptr(r), _stream()))
        return r

    def jvp(self, state, v, *, return_residual: bool = False, precision: int = 64):
        """``J v``; ``precision=32`` evaluates the tangent pass in fp32 arithmetic
        (``fv_jvp_f32``: ~1e-6 relative, for the Krylov operator of a mixed-precision Newton)."""
        s, vv = self._vec(state), self._vec(v)
        jv = torch.empty_like(s)
        if precision == 32:
            if return_residual:
                raise ValueError("the fp32 JVP returns no residual")
            check(lib().fv_jvp_f32(self._h, ptr(s), ptr(vv), ptr(jv), _stream()))
            return jv
        if precision != 64:
            raise ValueError(f"precision must be 64 or 32, got {precision}")
        r = torch.empty_like(s) if return_residual else None
        check(lib().fv_jvp(self._h, ptr(s), ptr(vv), ptr(r), ptr(jv), _stream()))
        return (r, jv) if return_residual else jv

    def linearise(self, state, out: torch.Tensor | None = None) -> torch.Tensor:
        """``R(state)``, holding the evaluation's face intermediates, gradients, residual and (SST)
        the off-wall closure and source tangents as linear forms, for :meth:`jvp_linearised`
        (``fv_linearise``; first-order upwind advection only)."""
        s = self._vec(state)
        r = torch.empty_like(s) if out is None else out
        check(lib().fv_linearise(self._h, ptr(s), ptr(r), _stream()))
        return r

    def jvp_linearised(self, state, v) -> torch.Tensor:
        """``J(state) v`` at the state last passed to :meth:`linearise` (``fv_jvp_linearised``:
        the interior faces' flux, coefficient and compact-gradient stages, the off-wall closure and
        the face sums as tangents from the held linearisation; the same product as :meth:`jvp`
        within rounding)."""
        s, vv = self._vec(state), self._vec(v)
        jv = torch.empty_like(s)
        check(lib().fv_jvp_linearised(self._h, ptr(s), ptr(vv), 0, ptr(jv), _stream()))
        return jv

    def hold_forward(self, state, out: torch.Tensor | None = None) -> torch.Tensor:
        """``R(state)``, holding the VJP's forward pass for :meth:`vjp_held` (``fv_hold_forward``)."""
        s = self._vec(state)
        r = torch.empty_like(s) if out is None else out
        check(lib().fv_hold_forward(self._h, ptr(s), ptr(r), _stream()))
        return r

    def vjp_held(self, state, w) -> torch.Tensor:
        """``w^T J(state)`` by the adjoint stages alone, at the state of the held forward pass
        (``fv_vjp_held``; bitwise :meth:`vjp`)."""
        s, ww = self._vec(state), self._vec(w)
        out = torch.empty_like(s)
        check(lib().fv_vjp_held(self._h, ptr(s), ptr(ww), ptr(out), _stream()))
        return out

    def node_vjp(self, state, w) -> torch.Tensor:
        """``d/dnodes (w . R(state, nodes))``, shape ``(n_nodes, dim)`` (the mesh-coordinate
        adjoint; compact gradient scheme)."""
        s, ww = self._vec(state), self._vec(w)
        mesh = self.dmesh.mesh
        out = torch.empty(mesh.n_nodes, mesh.dim, dtype=torch.float64, device="cuda")
        check(lib().fv_node_vjp(self._h, ptr(s), ptr(ww), ptr(out), _stream()))
        return out

    def autotune(self, state, w) -> int:
        """Pick the stage kernels' block sizes by timing the residual + VJP step, each stage its own
        fastest (``fv_case_autotune``); returns the fastest uniform size."""
        s, ww = self._vec(state), self._vec(w)
        out = torch.empty_like(s)
        best = ctypes.c_int(0)
        check(lib().fv_case_autotune(self._h, ptr(s), ptr(ww), ptr(out), _stream(),
                                     ctypes.byref(best)))
        return int(best.value)

    def set_persistent(self, enable: bool = True, block: int = 128, chunk: int = 1) -> None:
        """Evaluate residual + VJP as one persistent cooperative launch (``fv_case_set_persistent``;
        compact gradients, first-order upwind)."""
        check(lib().fv_case_set_persistent(self._h, int(bool(enable)), int(block), int(chunk)))

    def autotune_persistent(self, state, w) -> tuple[int, int, float]:
        """``(block, chunk, ms)`` of the fastest persistent launch at ``state`` / ``w``."""
        s, ww = self._vec(state), self._vec(w)
        out = torch.empty_like(s)
        b, c, t = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_float(0.0)
        check(lib().fv_case_autotune_persistent(self._h, ptr(s), ptr(ww), ptr(out), _stream(),
                                                ctypes.byref(b), ctypes.byref(c),
                                                ctypes.byref(t)))
        return b.value, c.value, t.value

    def set_block_size(self, threads: int) -> None:
        check(lib().fv_case_set_block_size(self._h, int(threads)))

    def block_sizes(self) -> list[int]:
        """Threads per block of each stage kernel (``fv_case_block_sizes``; the stages of
        :attr:`STAGES`)."""
        out = (ctypes.c_int * len(self.STAGES))()
        check(lib().fv_case_block_sizes(self._h, out, len(self.STAGES)))
        return list(out)

    def set_cell_order(self, coherent: bool = True) -> int:
        """Thread-to-cell order of the cell-centric stages (``fv_case_set_cell_order``): grouped by
        face-list pattern so that warps do not diverge (default), or natural.  Bitwise the same
        results; returns the number of distinct patterns."""
        n = ctypes.c_int(0)
        check(lib().fv_case_set_cell_order(self._h, int(bool(coherent)), ctypes.byref(n)))
        return n.value

    def functional_weights(self, spec: dict) -> torch.Tensor:
        """Weights of a face-flux functional: ``spec = {patch: {field: weight}}`` puts ``weight``
        on the ``field`` flux of every face of ``patch`` (fields: 0..dim-1 momentum, dim
        continuity, dim+1 / dim+2 k / omega)."""
        mesh = self.dmesh.mesh
        nfld = self.n_unknowns // self.n_cells
        w = np.zeros((nfld, mesh.n_faces))
        for patch, fields in spec.items():
            faces = np.asarray(mesh.patches[patch], dtype=np.int64)
            for q, val in fields.items():
                w[int(q), faces] = float(val)
        return torch.tensor(w, device="cuda")

    def face_functional(self, state, weights, *, viscous_only: bool = False, params: bool = True,
                        nodes: bool = True) -> dict:
        """``J = sum w . FL`` (less the boundary pressure part with ``viscous_only``): its value,
        ``dJ/dstate``, ``dJ/d(mu, inlet_scale)`` and ``dJ/dnodes`` at fixed state."""
        s = self._vec(state)
        w = torch.as_tensor(weights, dtype=torch.float64, device="cuda").contiguous()
        mesh = self.dmesh.mesh
        value = torch.empty(1, dtype=torch.float64, device="cuda")
        dstate = torch.empty_like(s)
        dparams = torch.empty(2, dtype=torch.float64, device="cuda") if params else None
        dnodes = (torch.empty(mesh.n_nodes, mesh.dim, dtype=torch.float64, device="cuda")
                  if nodes else None)
        check(lib().fv_face_functional(self._h, ptr(s), ptr(w), int(viscous_only), ptr(value),
                                       ptr(dstate), ptr(dparams), ptr(dnodes), _stream()))
        return {"value": float(value), "dstate": dstate, "dparams": dparams, "dnodes": dnodes}

    def jvp_batch(self, state, vs) -> torch.Tensor:
        """``J(state) v_i`` for every row of the ``(k, n)`` seed block ``vs``."""
        s = self._vec(state)
        v = torch.as_tensor(vs, dtype=torch.float64, device="cuda").contiguous()
        if v.dim() != 2 or v.shape[1] != self.n_unknowns:
            raise ValueError(f"expected seeds of shape (k, {self.n_unknowns}), got {tuple(v.shape)}")
        out = torch.empty_like(v)
        check(lib().fv_jvp_batch(self._h, ptr(s), ptr(v), int(v.shape[0]), ptr(out), _stream()))
        return out

    def jvp_shift(self, state, v, shift) -> torch.Tensor:
        s, vv, sh = self._vec(state), self._vec(v), self._vec(shift)
        jv = torch.empty_like(s)
        check(lib().fv_jvp_shift(self._h, ptr(s), ptr(vv), ptr(sh), ptr(jv), _stream()))
        return jv

    def vjp(self, state, w, *, return_residual: bool = False):
        """``J(state)^T w`` (hand-written adjoint kernels); optionally also ``R(state)``."""
        s, ww = self._vec(state), self._vec(w)
        g = torch.empty_like(s)
        r = torch.empty_like(s) if return_residual else None
        check(lib().fv_vjp(self._h, ptr(s), ptr(ww), ptr(r), ptr(g), _stream()))
        return (r, g) if return_residual else g

    def param_vjp(self, state, w) -> torch.Tensor:
        """``(w . dR/dmu, w . dR/d inlet_scale)`` as a 2-vector on the device."""
        s, ww = self._vec(state), self._vec(w)
        out = torch.empty(2, dtype=torch.float64, device="cuda")
        check(lib().fv_param_vjp(self._h, ptr(s), ptr(ww), ptr(out), _stream()))
        return out

    def param_jvp(self, state):
        """``(dR/dmu, dR/d inlet_scale)`` at ``state``."""
        s = self._vec(state)
        a, b = torch.empty_like(s), torch.empty_like(s)
        check(lib().fv_param_jvp(self._h, ptr(s), ptr(a), ptr(b), _stream()))
        return a, b

    STAGES = ("grad", "closure", "apcoef", "dcoeff", "flux", "sum",
              "a_sum", "a_flux", "a_apcoef", "a_closure", "a_grad")

    def profile_begin(self, max_runs: int) -> None:
        check(lib().fv_case_profile_begin(self._h, int(max_runs)))

    def profile_end(self) -> tuple[dict, int]:
        """Summed per-stage milliseconds of the profiled runs, and the run count."""
        ms = (ctypes.c_float * len(self.STAGES))()
        n = ctypes.c_int(0)
        check(lib().fv_case_profile_end(self._h, ms, len(self.STAGES), ctypes.byref(n)))
        return {k: float(ms[i]) for i, k in enumerate(self.STAGES)}, int(n.value)

    def pattern_plan(self, key, build):
        """A product of the mesh's connectivity alone -- a Jacobian sparsity pattern, a colouring
        order, an aggregation hierarchy's host plan -- built by ``build()`` on first use and kept
        for every later solve on this case, as the mesh geometry is (moving the nodes keeps it).
        The reference hoists the same pattern-dependent structures out of its refreshes and
        solves (``aquaflux/solve/amg_preconditioner.py:740-760``: the probe ``plan`` and gather
        ``structure``, built once)."""
        plans = self.__dict__.setdefault("_pattern_plans", {})
        if key not in plans:
            plans[key] = build()
        return plans[key]

    def set_nodes(self, nodes: torch.Tensor) -> None:
        """Move the mesh nodes: recompute the geometry and (turbulent case) the SST wall
        distance to each cell's nearest wall face, that face held fixed."""
        self.dmesh.set_nodes(nodes)
        check(lib().fv_case_refresh_geometry(self._h, _stream()))

    def set_wall_distance(self, distance) -> None:
        """Replace the SST wall distance (per cell) and recompute its gradient."""
        d = torch.as_tensor(distance, dtype=torch.float64, device="cuda").reshape(-1)
        if d.numel() != self.n_cells:
            raise ValueError(f"expected {self.n_cells} wall distances, got {d.numel()}")
        check(lib().fv_case_set_wall_distance(self._h, ptr(d.contiguous()), _stream()))

    def wall_distance(self):
        C, D = self.n_cells, self.dim
        d = torch.empty(C, dtype=torch.float64, device="cuda")
        g = torch.empty(C, D, dtype=torch.float64, device="cuda")
        check(lib().fv_case_wall_distance(self._h, ptr(d), ptr(g), _stream()))
        return d, g

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().fv_case_destroy(h)
            except Exception:
                pass
