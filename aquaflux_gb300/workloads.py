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
                           pressure_pin=self.pressure_pin, sst=self.sst, gradient=self.gradient)


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
              seed: int = 0, renumber: bool = True) -> Workload:
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    extent = (2.0, 1.0, 1.0)
    m = fm.structured_grid_3d(nx, ny, nz, *extent)
    m = m.with_nodes(fm.bump_channel_nodes_3d((nx, ny, nz), extent, 0.1, 0.1, seed))
    if renumber:
        m = fm.permute_cells(m, fm.random_permutation(m.n_cells, seed))
        m = fm.permute_cells(m, rcm_permutation(m))
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
