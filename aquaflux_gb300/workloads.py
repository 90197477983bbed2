"""Seeded synthetic workloads standing in for the benchmark configurations.

There is no public dataset behind these cases: each is a structured mesh with seeded node
perturbations and a case description, built the same way on every machine.

* :func:`cavity` -- lid-driven cavity, laminar (u, v, p), ``structured_grid_2d(n, n)``, lid u=1,
  mu = 0.01, rho = 1, pressure pinned in cell 0 (the reference's ``tests/integration/test_cavity.py``
  setup); 64 x 64 is the 4,096-cell configuration.
* :func:`channel3d` -- 3D channel with a seeded Gaussian bump (height 0.1) on the lower wall,
  interior nodes jittered +-0.1 of the spacing, cells randomly permuted then relabelled by reverse
  Cuthill-McKee; coupled (u, v, w, p) + k-omega SST, velocity inlet (u = 1, turbulence intensity
  5 %, length scale 0.07), pressure outlet, four no-slip walls.  128^3 is the 2,097,152-cell case
  (6,340,608 faces).
* :func:`backward_step` -- 2D backward-facing step (:func:`aquaflux_gb300.mesh.backward_step_2d`:
  inlet height h = 1, step 0.5 h, expansion ratio 1.5, a 30h x 1.5h domain, ~200k quads graded to
  the walls, interior nodes jittered +-0.15 of the local spacing), coupled (u, v, p) + k-omega SST
  at Re_h = 5e4 (nu = 2e-5, inlet u = 1, intensity 5 %), corrected Green-Gauss gradients by four
  swept sweeps.
* :func:`batched_channels` -- the batched calibration sweep: 64 independent 2D laminar channels
  (2 x 1, inlet / outlet / two walls) of uneven size n x n, n log-uniform in [32, 256], viscosity
  log-uniform in [1e-3, 1e-1], inlet velocity uniform in [0.5, 2], held side by side in one
  disjoint-union mesh (one launch per stage for all instances) with a per-cell viscosity field.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import mesh as fm

BETA_STAR, KAPPA = 0.09, 0.41


def inlet_k(velocity_magnitude: float, intensity: float) -> float:
    """``1.5 (U I)^2`` (``aquaflux/turbulence/boundary.py:423-438``)."""
    return 1.5 * (velocity_magnitude * intensity) ** 2


def inlet_omega(k: float, length_scale: float) -> float:
    """``sqrt(k) / (beta_star^0.25 l)`` (``aquaflux/turbulence/boundary.py:470-488``)."""
    return float(np.sqrt(k) / (BETA_STAR ** 0.25 * length_scale))


@dataclasses.dataclass
class Workload:
    name: str
    mesh: fm.MeshData
    mu: float
    rho: float
    flow_bc: dict
    pressure_pin: int | None
    sst: dict | None
    k_in: float = 0.0
    omega_in: float = 0.0
    gradient: dict | None = None
    advection: dict | None = None
    k_transform: str = "direct"      # solved variable of k: "direct" or "log" (k = exp(w_k))
    omega_transform: str = "direct"  # ... of omega (LogScalars, omega = exp(w))
    scalar_advection: object = None  # k / omega advection when not the momentum scheme

    @property
    def n_unknowns(self) -> int:
        return (self.mesh.dim + (3 if self.sst else 1)) * self.mesh.n_cells

    def initial_state(self, seed: int = 0, noise: float = 0.0) -> np.ndarray:
        """A smooth admissible state: plug flow along x (zero in a closed cavity), inlet k / omega."""
        rng = np.random.default_rng(seed)
        n, d = self.mesh.n_cells, self.mesh.dim
        u = np.zeros((d, n))
        if self.sst is not None:
            u[0] = 1.0
        p = np.zeros(n)
        parts = [u.reshape(-1), p]
        if self.sst is not None:
            parts += [np.full(n, self.k_in), np.full(n, self.omega_in)]
        s = np.concatenate(parts)
        if noise:
            s = s * (1.0 + noise * rng.standard_normal(s.size)) + noise * 0.1 * rng.standard_normal(s.size) * (s == 0)
        return s

    def device_case(self):
        from . import fv

        dm = fv.DeviceMesh(self.mesh)
        return fv.FlowCase(dm, mu=self.mu, rho=self.rho, flow_bc=self.flow_bc,
                           pressure_pin=self.pressure_pin, sst=self.sst, gradient=self.gradient,
                           advection=self.advection, k_transform=self.k_transform,
                           omega_transform=self.omega_transform,
                           scalar_advection=self.scalar_advection)


def cavity(n: int = 64, mu: float = 0.01, lid: float = 1.0) -> Workload:
    m = fm.structured_grid_2d(n, n)
    bc = {"top": ("moving", (lid, 0.0)), "bottom": ("wall",), "left": ("wall",), "right": ("wall",)}
    return Workload(f"cavity{n}", m, mu, 1.0, bc, 0, None)


def rcm_permutation(mesh: fm.MeshData) -> np.ndarray:
    """``ReverseCuthillMcKee.permutation`` (``aquaflux/mesh/reorder.py:147-159``): scipy's RCM on the
    symmetric cell graph, returned as ``perm[old] = new``."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import reverse_cuthill_mckee

    ip, ix = fm.cell_adjacency_csr(mesh)
    g = sp.csr_matrix((np.ones(ix.size), ix, ip), shape=(mesh.n_cells, mesh.n_cells))
    old_order = reverse_cuthill_mckee(g, symmetric_mode=True)
    return np.argsort(old_order)


def channel3d(nx: int = 128, ny: int | None = None, nz: int | None = None, *, nu: float = 5e-4,
              seed: int = 0, renumber: bool | str = True) -> Workload:
    """``renumber``: True or ``"gpu"`` -- random relabelling, then reverse Cuthill-McKee computed
    on the GPU (:mod:`aquaflux_gb300.reorder`); ``"host"`` -- the same permutation by scipy on
    the host (the reference's own call; for machines without a GPU); False -- natural order."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    extent = (2.0, 1.0, 1.0)
    m = fm.structured_grid_3d(nx, ny, nz, *extent)
    m = m.with_nodes(fm.bump_channel_nodes_3d((nx, ny, nz), extent, 0.1, 0.1, seed))
    if renumber not in (True, False, "gpu", "host"):
        raise ValueError(f"renumber must be True, False, 'gpu' or 'host', got {renumber!r}")
    if renumber:
        m = fm.permute_cells(m, fm.random_permutation(m.n_cells, seed))
        if renumber == "host":
            perm = rcm_permutation(m)
        else:
            from .reorder import mesh_rcm_permutation

            perm = mesh_rcm_permutation(m)
        m = fm.permute_cells(m, perm)
    k_in = inlet_k(1.0, 0.05)
    w_in = inlet_omega(k_in, 0.07)
    walls = ["bottom", "top", "back", "front"]
    flow_bc = {"left": ("inlet", (1.0, 0.0, 0.0)), "right": ("outlet", 0.0)}
    flow_bc.update({w: ("wall",) for w in walls})
    kb = {"left": ("dirichlet", k_in), "right": ("zerograd",)}
    kb.update({w: ("dirichlet", 0.0) for w in walls})
    wb = {"left": ("dirichlet", w_in), "right": ("zerograd",)}
    wb.update({w: ("zerograd",) for w in walls})
    sst = {"walls": walls, "k": kb, "omega": wb}
    return Workload(f"channel3d_{nx}x{ny}x{nz}_sst", m, nu, 1.0, flow_bc, None, sst, k_in, w_in)


def backward_step(*, n_step: int = 48, n_channel: int = 96, n_upstream: int = 120,
                  n_downstream: int = 1300, nu: float = 2e-5, seed: int = 0,
                  sweeps: int = 4) -> Workload:
    m = fm.backward_step_2d(n_step=n_step, n_channel=n_channel, n_upstream=n_upstream,
                            n_downstream=n_downstream, seed=seed)
    k_in = inlet_k(1.0, 0.05)
    w_in = inlet_omega(k_in, 0.07)
    walls = ["bottom", "top", "step"]
    flow_bc = {"inlet": ("inlet", (1.0, 0.0)), "outlet": ("outlet", 0.0)}
    flow_bc.update({w: ("wall",) for w in walls})
    kb = {"inlet": ("dirichlet", k_in), "outlet": ("zerograd",)}
    kb.update({w: ("dirichlet", 0.0) for w in walls})
    wb = {"inlet": ("dirichlet", w_in), "outlet": ("zerograd",)}
    wb.update({w: ("zerograd",) for w in walls})
    sst = {"walls": walls, "k": kb, "omega": wb}
    return Workload(f"backward_step_{m.n_cells}_sst", m, nu, 1.0, flow_bc, None, sst, k_in, w_in,
                    gradient={"sweeps": sweeps, "relaxation": 1.0} if sweeps else None)


@dataclasses.dataclass
class BatchedWorkload:
    workload: Workload      # the disjoint union (laminar, per-cell viscosity)
    offsets: np.ndarray     # (n_instances + 1) cell offsets of the instances
    mu: np.ndarray          # per instance
    velocity: np.ndarray    # per-instance inlet velocity
    sizes: np.ndarray       # cells per axis of each instance

    @property
    def n_instances(self) -> int:
        return int(self.mu.size)

    def initial_state(self) -> np.ndarray:
        """Plug flow at each instance's inlet velocity, zero pressure."""
        m = self.workload.mesh
        n = m.n_cells
        u = np.zeros((m.dim + 1, n))
        u[0] = np.repeat(self.velocity, np.diff(self.offsets))
        return u.reshape(-1)

    def outlet_weights(self, areas: np.ndarray) -> np.ndarray:
        """``g`` with ``g . state`` restricted to instance i equal to its mean outlet velocity
        ``sum_f A_f u_P(f) / sum_f A_f`` over the outlet faces (the outlet boundary value is the
        owner's velocity)."""
        m = self.workload.mesh
        g = np.zeros((m.dim + 1) * m.n_cells)
        for i in range(self.n_instances):
            faces = np.asarray(m.patches[f"{i}:right"], dtype=np.int64)
            a = areas[faces]
            np.add.at(g, m.owner[faces], a / a.sum())
        return g


def batched_channels(n_instances: int = 64, *, n_min: int = 32, n_max: int = 256,
                     seed: int = 0) -> BatchedWorkload:
    rng = np.random.default_rng(seed)
    sizes = np.rint(np.exp(rng.uniform(np.log(n_min), np.log(n_max), n_instances))).astype(int)
    mu = np.exp(rng.uniform(np.log(1e-3), np.log(1e-1), n_instances))
    vel = rng.uniform(0.5, 2.0, n_instances)
    meshes = [fm.structured_grid_2d(int(n), int(n), 2.0, 1.0) for n in sizes]
    union, offsets = fm.disjoint_union(meshes)
    flow_bc = {}
    for i in range(n_instances):
        flow_bc[f"{i}:left"] = ("inlet", (float(vel[i]), 0.0))
        flow_bc[f"{i}:right"] = ("outlet", 0.0)
        flow_bc[f"{i}:bottom"] = ("wall",)
        flow_bc[f"{i}:top"] = ("wall",)
    mu_cell = np.repeat(mu, np.diff(offsets))
    wl = Workload(f"batched_channels_{n_instances}_{union.n_cells}", union, mu_cell, 1.0,
                  flow_bc, None, None)
    return BatchedWorkload(wl, offsets, mu, vel, sizes)
