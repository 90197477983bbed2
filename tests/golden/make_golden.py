"""Generate the golden vectors in this folder by running the reference package itself.

Run from the repository root, in a container that has the reference source checked out:

    python tests/golden/make_golden.py <path of the reference checkout>

JAX is not installed there, so the reference's forward code runs on :mod:`refshim` (numpy float64
stand-ins for ``jax.numpy`` / ``equinox``).  Everything written here is produced by the reference's
own functions:

* mesh topology and geometry: ``aquaflux.mesh.structured_grid_2d/3d`` and ``Mesh.geometry()``
  (``aquaflux/mesh/structured.py:155-375``, ``aquaflux/mesh/mesh.py:341-387``);
* residuals: ``MomentumContinuity.residual`` (``aquaflux/flow/momentum.py:880``) and
  ``CoupledRANS.residual`` (``aquaflux/turbulence/coupled.py:437``), plus intermediate fields from
  ``MomentumContinuity.flow_fields`` (``momentum.py:822``);
* JVP goldens: central finite differences of those reference residuals;
* ILU(0): the reference's pure-Python twin (``aquaflux/solve/ilu0.py:76-150``) on the fixture
  operator of ``tests/unit/test_ilu0.py:17-37``.

The only inputs this script invents are node coordinates (seeded jitter and a Gaussian bump) and the
seeded states; the same recipes are restated in ``aquaflux_gb300.mesh`` so the GPU tests rebuild
identical meshes without the reference.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import refshim  # noqa: E402

refshim.install()

if len(sys.argv) < 2:
    sys.exit("usage: make_golden.py <path of the reference checkout>")
REF = sys.argv[1]
sys.path.insert(0, REF)
sys.path.insert(0, os.path.join(REF, "tests"))

import jax.numpy as jnp  # noqa: E402  (the shim)
from aquaflux.boundary import BoundaryConditions, Dirichlet, ZeroGradient  # noqa: E402
from aquaflux.discretization import FirstOrderUpwind, LimitedUpwind  # noqa: E402
from aquaflux.schemes.limiter import VenkatakrishnanLimiter  # noqa: E402
from aquaflux.flow import (  # noqa: E402
    MomentumContinuity,
    MovingWall,
    NoSlipWall,
    PressureOutlet,
    VelocityInlet,
)
from aquaflux.mesh import graded_nodes, structured_grid_2d, structured_grid_3d  # noqa: E402
from aquaflux.properties import Constant, PropertyModel  # noqa: E402
from aquaflux.schemes import CompactGreenGauss, CorrectedGreenGauss  # noqa: E402
from aquaflux.schemes.gradient import SweptGradientSolve  # noqa: E402
from aquaflux.solve import ilu0 as ref_ilu0  # noqa: E402
from aquaflux.turbulence import SSTModel, SSTTurbulence, inlet_k, inlet_omega  # noqa: E402
from aquaflux.turbulence.coupled import CoupledRANS, LogScalars  # noqa: E402

sys.path.insert(0, os.path.join(REF, "tests", "unit"))

# The node-coordinate recipes live in the package (restated there for the GPU machine); importing
# them here guarantees that the fixtures and the GPU tests see the same coordinates.
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from aquaflux_gb300.mesh import bump_channel_nodes_3d, jitter_interior_nodes  # noqa: E402


def _with_nodes(mesh, nodes):
    return refshim._tree_at(lambda m: m.node_coords, mesh, jnp.asarray(nodes))


def _mesh_arrays(prefix, mesh, geom):
    fc = mesh.face_cells
    fn = mesh.face_nodes
    out = {
        f"{prefix}nodes": np.asarray(mesh.node_coords),
        f"{prefix}owner": np.asarray(fc.owner).astype(np.int32),
        f"{prefix}neighbour": np.asarray(fc.neighbour).astype(np.int32),
        f"{prefix}fn_offsets": np.asarray(fn.offsets).astype(np.int32),
        f"{prefix}fn_indices": np.asarray(fn.face_node_indices).astype(np.int32),
        f"{prefix}area": np.asarray(geom.face.area),
        f"{prefix}normal": np.asarray(geom.face.normal),
        f"{prefix}face_centroid": np.asarray(geom.face.centroid),
        f"{prefix}volume": np.asarray(geom.cell.volume),
        f"{prefix}cell_centroid": np.asarray(geom.cell.centroid),
    }
    patches = mesh.face_patches
    for name in patches.names:
        out[f"{prefix}patch_{name}"] = np.asarray(patches.indices(name)).astype(np.int32)
    return out


def _fd_jvp(fn, state, direction, h):
    return (np.asarray(fn(jnp.asarray(state + h * direction)))
            - np.asarray(fn(jnp.asarray(state - h * direction)))) / (2.0 * h)


# --------------------------------------------------------------------------- meshes
def mesh_cases():
    out = {}
    m = structured_grid_2d(5, 4, lx=2.0, ly=1.0, named_boundaries=True)
    m = _with_nodes(m, jitter_interior_nodes(np.asarray(m.node_coords), (5, 4), (2.0, 1.0), 0.15, 3))
    out.update(_mesh_arrays("m2d_", m, m.geometry()))
    m = structured_grid_3d(4, 3, 3, lx=2.0, ly=1.0, lz=1.0, named_boundaries=True)
    nodes = bump_channel_nodes_3d((4, 3, 3), (2.0, 1.0, 1.0), bump_height=0.1, jitter=0.1, seed=5)
    m = _with_nodes(m, nodes)
    out.update(_mesh_arrays("m3d_", m, m.geometry()))
    yn = graded_nodes(6, 1.0, 1.3)
    m = structured_grid_2d(7, 6, lx=3.0, ly=1.0, named_boundaries=True, y_nodes=yn)
    out.update(_mesh_arrays("mgr_", m, m.geometry()))
    out["mgr_y_nodes"] = np.asarray(yn)
    return out


# --------------------------------------------------------------------------- laminar flow
def _cavity(n, perturb=0.0, seed=0, mu=0.01, scheme=None, advection=None):
    mesh = structured_grid_2d(n, n, lx=1.0, ly=1.0, named_boundaries=True)
    if perturb:
        mesh = _with_nodes(mesh, jitter_interior_nodes(np.asarray(mesh.node_coords), (n, n),
                                                       (1.0, 1.0), perturb, seed))
    geom = mesh.geometry()
    asm = MomentumContinuity.build(
        mesh, geom, PropertyModel({"viscosity": Constant(mu), "density": Constant(1.0)}),
        scheme or CompactGreenGauss(),
        BoundaryConditions({"top": MovingWall(velocity=(1.0, 0.0)), "bottom": NoSlipWall(),
                            "left": NoSlipWall(), "right": NoSlipWall()}),
        advection_scheme=advection or FirstOrderUpwind(), pressure_pin=0)
    return mesh, geom, asm


def _laminar_channel3d(shape, mu=0.02, rho=1.0, u_in=1.0):
    nx, ny, nz = shape
    mesh = structured_grid_3d(nx, ny, nz, lx=2.0, ly=1.0, lz=1.0, named_boundaries=True)
    mesh = _with_nodes(mesh, bump_channel_nodes_3d(shape, (2.0, 1.0, 1.0), 0.1, 0.1, 7))
    geom = mesh.geometry()
    bcs = {"left": VelocityInlet(velocity=(u_in, 0.0, 0.0)), "right": PressureOutlet(pressure=0.0),
           "bottom": NoSlipWall(), "top": NoSlipWall(), "back": NoSlipWall(), "front": NoSlipWall()}
    asm = MomentumContinuity.build(
        mesh, geom, PropertyModel({"viscosity": Constant(mu), "density": Constant(rho)}),
        CompactGreenGauss(), BoundaryConditions(bcs), advection_scheme=FirstOrderUpwind())
    return mesh, geom, asm


def _flow_fields(prefix, asm, state):
    f = asm.flow_fields(jnp.asarray(state))
    a_p = asm.momentum_matrix_diagonal(f.velocity_fields.velocity, f.velocity_fields.gradient)
    return {
        f"{prefix}grad_u": np.asarray(f.velocity_fields.gradient),
        f"{prefix}grad_p": np.asarray(f.grad_pressure),
        f"{prefix}mdot": np.asarray(f.mdot),
        f"{prefix}a_p": np.asarray(a_p)[:, 0],
        f"{prefix}bvel": np.asarray(f.velocity_fields.boundary_velocity),
        f"{prefix}bp": np.asarray(f.boundary_pressure),
    }


def laminar_cases():
    out = {}
    rng = np.random.default_rng(11)
    # 8x8 cavity (structured): zero state + two random states (+ FD JVP for the second).
    mesh, geom, asm = _cavity(8)
    out.update(_mesh_arrays("cav8_", mesh, geom))
    states = [np.zeros(3 * 64), rng.standard_normal(3 * 64) * 0.3, rng.standard_normal(3 * 64)]
    out["cav8_states"] = np.stack(states)
    out["cav8_residuals"] = np.stack([np.asarray(asm.residual(jnp.asarray(s))) for s in states])
    out.update(_flow_fields("cav8_s1_", asm, states[1]))
    v = rng.standard_normal(3 * 64)
    out["cav8_jvp_dir"] = v
    out["cav8_jvp_fd"] = _fd_jvp(asm.residual, states[1], v, 1e-6)
    # Config-1 size (64x64, structured): zero state and one random state.
    mesh, geom, asm = _cavity(64)
    s = rng.standard_normal(3 * 4096) * 0.2
    out["cav64_states"] = np.stack([np.zeros(3 * 4096), s])
    out["cav64_residuals"] = np.stack([np.asarray(asm.residual(jnp.asarray(x)))
                                       for x in out["cav64_states"]])
    # Jittered 10x10 cavity (non-orthogonal corrections active).
    mesh, geom, asm = _cavity(10, perturb=0.15, seed=0)
    out.update(_mesh_arrays("cavj_", mesh, geom))
    states = [rng.standard_normal(300) * 0.3, rng.standard_normal(300)]
    out["cavj_states"] = np.stack(states)
    out["cavj_residuals"] = np.stack([np.asarray(asm.residual(jnp.asarray(s))) for s in states])
    out.update(_flow_fields("cavj_s0_", asm, states[0]))
    v = rng.standard_normal(300)
    out["cavj_jvp_dir"] = v
    out["cavj_jvp_fd"] = _fd_jvp(asm.residual, states[0], v, 1e-6)
    # 3D laminar channel with a bump, inlet/outlet/walls.
    mesh, geom, asm = _laminar_channel3d((4, 3, 3))
    out.update(_mesh_arrays("lam3_", mesh, geom))
    n = mesh.n_cells
    states = []
    for _ in range(2):
        u = 1.0 + 0.3 * rng.standard_normal(n)
        states.append(np.concatenate([u, 0.2 * rng.standard_normal(2 * n), 0.1 * rng.standard_normal(n)]))
    out["lam3_states"] = np.stack(states)
    out["lam3_residuals"] = np.stack([np.asarray(asm.residual(jnp.asarray(s))) for s in states])
    out.update(_flow_fields("lam3_s0_", asm, states[0]))
    v = rng.standard_normal(4 * n)
    out["lam3_jvp_dir"] = v
    out["lam3_jvp_fd"] = _fd_jvp(asm.residual, states[0], v, 1e-6)
    return out


# --------------------------------------------------------------------------- k-omega SST
def _rans(mesh, geom, dim, nu, u_in, walls, inlet="left", outlet="right", intensity=0.05,
          length_scale=0.07, scheme=None, advection=None, k_transform=None, omega_transform=None,
          scalar_advection=None, k_wall=None):
    scheme = scheme or CompactGreenGauss()
    advection = advection or FirstOrderUpwind()
    rho = 1.0
    model = SSTModel()
    k_in = float(inlet_k(jnp.array(u_in), intensity))
    omega_in = float(inlet_omega(jnp.array(k_in), length_scale, model))
    vel = (u_in,) + (0.0,) * (dim - 1)
    flow_bc = {inlet: VelocityInlet(velocity=vel), outlet: PressureOutlet(pressure=0.0)}
    flow_bc.update({w: NoSlipWall() for w in walls})
    k_bc = {inlet: Dirichlet(k_in), outlet: ZeroGradient()}
    k_bc.update({w: (k_wall or Dirichlet(0.0)) for w in walls})
    w_bc = {inlet: Dirichlet(omega_in), outlet: ZeroGradient()}
    w_bc.update({w: ZeroGradient() for w in walls})
    momentum = MomentumContinuity.build(
        mesh, geom, PropertyModel({"viscosity": Constant(rho * nu), "density": Constant(rho)}),
        scheme, BoundaryConditions(flow_bc), advection_scheme=advection)
    turb = SSTTurbulence.build(
        model, mesh, geom, scheme, scalar_advection or advection, density=rho,
        molecular_viscosity=jnp.full(mesh.n_cells, nu), wall_patches=list(walls),
        k_boundary=BoundaryConditions(k_bc), omega_boundary=BoundaryConditions(w_bc))
    return (CoupledRANS.build(momentum, turb, k_transform=k_transform,
                              omega_transform=omega_transform), turb, k_in, omega_in)


def _rans_states(rng, n, dim, k_in, omega_in, count, negative_k=False):
    states = []
    for i in range(count):
        u = 1.0 + 0.3 * rng.standard_normal(n)
        rest = 0.2 * rng.standard_normal((dim - 1) * n)
        p = 0.1 * rng.standard_normal(n)
        k = k_in * (0.3 + rng.random(n)) * (1.0 + 20.0 * rng.random(n))
        om = omega_in * (0.3 + rng.random(n)) * (1.0 + 5.0 * rng.random(n))
        if negative_k and i == count - 1:
            k[rng.choice(n, size=max(1, n // 10), replace=False)] *= -0.5
        states.append(np.concatenate([u, rest, p, k, om]))
    return states


def sst_cases():
    out = {}
    rng = np.random.default_rng(23)
    # 2D graded, jittered channel (the backward-step configuration's physics at fixture size).
    nx, ny = 12, 8
    yn = graded_nodes(ny, 1.0, 1.2)
    mesh = structured_grid_2d(nx, ny, lx=4.0, ly=1.0, named_boundaries=True, y_nodes=yn)
    mesh = _with_nodes(mesh, jitter_interior_nodes(np.asarray(mesh.node_coords), (nx, ny),
                                                   (4.0, 1.0), 0.1, 4))
    geom = mesh.geometry()
    coupled, turb, k_in, omega_in = _rans(mesh, geom, 2, 2e-5, 1.0, ["bottom", "top"])
    out.update(_mesh_arrays("sst2_", mesh, geom))
    out["sst2_y_nodes"] = np.asarray(yn)
    out["sst2_wall_distance"] = np.asarray(turb.wall_distance)
    out["sst2_wall_distance_gradient"] = np.asarray(turb.wall_distance_gradient)
    out["sst2_inlet"] = np.array([k_in, omega_in])
    n = mesh.n_cells
    states = _rans_states(rng, n, 2, k_in, omega_in, 3, negative_k=True)
    out["sst2_states"] = np.stack(states)
    out["sst2_residuals"] = np.stack([np.asarray(coupled.residual(jnp.asarray(s))) for s in states])
    v = rng.standard_normal(5 * n)
    scale = np.abs(states[0]) + 1e-3
    out["sst2_jvp_dir"] = v * scale
    out["sst2_jvp_fd"] = _fd_jvp(coupled.residual, states[0], v * scale, 1e-7)
    # 3D duct with a bump.
    shape = (5, 4, 3)
    mesh = structured_grid_3d(*shape, lx=2.0, ly=1.0, lz=1.0, named_boundaries=True)
    mesh = _with_nodes(mesh, bump_channel_nodes_3d(shape, (2.0, 1.0, 1.0), 0.1, 0.1, 9))
    geom = mesh.geometry()
    walls = ["bottom", "top", "back", "front"]
    coupled, turb, k_in, omega_in = _rans(mesh, geom, 3, 1e-3, 1.0, walls)
    out.update(_mesh_arrays("sst3_", mesh, geom))
    out["sst3_wall_distance"] = np.asarray(turb.wall_distance)
    out["sst3_wall_distance_gradient"] = np.asarray(turb.wall_distance_gradient)
    out["sst3_inlet"] = np.array([k_in, omega_in])
    n = mesh.n_cells
    states = _rans_states(rng, n, 3, k_in, omega_in, 2)
    out["sst3_states"] = np.stack(states)
    out["sst3_residuals"] = np.stack([np.asarray(coupled.residual(jnp.asarray(s))) for s in states])
    v = rng.standard_normal(6 * n)
    scale = np.abs(states[0]) + 1e-3
    out["sst3_jvp_dir"] = v * scale
    out["sst3_jvp_fd"] = _fd_jvp(coupled.residual, states[0], v * scale, 1e-7)
    return out


# --------------------------------------------------------------------------- log-solved scalars
def logscalar_cases():
    """``CoupledRANS`` with ``LogScalars`` (``aquaflux/turbulence/coupled.py:178-207``): the state
    holds ``log omega`` (and ``log k`` in the 3D case); the near-wall omega rows are the log ratio
    (``LogRatioRow``, ``aquaflux/discretization/fixed_value.py:96-120``).  Same meshes and inlet
    conditions as the direct cases ``sst2_`` / ``sst3_``."""
    out = {}
    rng = np.random.default_rng(41)
    nx, ny = 12, 8
    yn = graded_nodes(ny, 1.0, 1.2)
    mesh = structured_grid_2d(nx, ny, lx=4.0, ly=1.0, named_boundaries=True, y_nodes=yn)
    mesh = _with_nodes(mesh, jitter_interior_nodes(np.asarray(mesh.node_coords), (nx, ny),
                                                   (4.0, 1.0), 0.1, 4))
    shape = (5, 4, 3)
    mesh3 = structured_grid_3d(*shape, lx=2.0, ly=1.0, lz=1.0, named_boundaries=True)
    mesh3 = _with_nodes(mesh3, bump_channel_nodes_3d(shape, (2.0, 1.0, 1.0), 0.1, 0.1, 9))
    for prefix, m, dim, nu, walls, log_k in (
            ("wsst2_", mesh, 2, 2e-5, ["bottom", "top"], False),
            ("bsst3_", mesh3, 3, 1e-3, ["bottom", "top", "back", "front"], True)):
        geom = m.geometry()
        coupled, turb, k_in, omega_in = _rans(
            m, geom, dim, nu, 1.0, walls, k_transform=LogScalars() if log_k else None,
            omega_transform=LogScalars())
        out.update(_mesh_arrays(prefix, m, geom))
        out[prefix + "wall_distance"] = np.asarray(turb.wall_distance)
        out[prefix + "wall_distance_gradient"] = np.asarray(turb.wall_distance_gradient)
        out[prefix + "inlet"] = np.array([k_in, omega_in])
        n = m.n_cells
        states = []
        for phys in _rans_states(rng, n, dim, k_in, omega_in, 2):
            solved = phys.copy()
            solved[(dim + 2) * n:] = np.log(phys[(dim + 2) * n:])
            if log_k:
                solved[(dim + 1) * n:(dim + 2) * n] = np.log(phys[(dim + 1) * n:(dim + 2) * n])
            states.append(solved)
        out[prefix + "states"] = np.stack(states)
        out[prefix + "residuals"] = np.stack([np.asarray(coupled.residual(jnp.asarray(s)))
                                              for s in states])
        v = rng.standard_normal((dim + 3) * n)
        scale = np.abs(states[0]) + 1e-3
        out[prefix + "jvp_dir"] = v * scale
        out[prefix + "jvp_fd"] = _fd_jvp(coupled.residual, states[0], v * scale, 1e-7)
    return out


# --------------------------------------------------------------------------- mixed schemes
def mixed_cases():
    """Momentum and k / omega on different advection schemes (``SSTTurbulence.build`` takes its
    own, ``aquaflux/turbulence/transport.py:266-312``): ``psst2_`` is the reference's backward-step
    validation configuration (``validation/pitzdaily_openfoam/compare.py:483-600``) at fixture
    size -- Venkatakrishnan-limited linear upwind momentum, first-order upwind k / omega, corrected
    Green-Gauss (4 sweeps), zero-gradient k on the walls, log omega; ``msst2_`` the reverse
    split (upwind momentum, limited scalars)."""
    out = {}
    rng = np.random.default_rng(53)
    nx, ny = 12, 8
    yn = graded_nodes(ny, 1.0, 1.2)
    mesh = structured_grid_2d(nx, ny, lx=4.0, ly=1.0, named_boundaries=True, y_nodes=yn)
    mesh = _with_nodes(mesh, jitter_interior_nodes(np.asarray(mesh.node_coords), (nx, ny),
                                                   (4.0, 1.0), 0.1, 4))
    geom = mesh.geometry()
    lim = LimitedUpwind(limiter=VenkatakrishnanLimiter(k=5.0))
    for prefix, kw, log_w in (
            ("psst2_", dict(advection=lim, scalar_advection=FirstOrderUpwind(),
                            scheme=_swept(4), k_wall=ZeroGradient()), True),
            ("msst2_", dict(advection=FirstOrderUpwind(), scalar_advection=lim), False)):
        coupled, turb, k_in, omega_in = _rans(mesh, geom, 2, 2e-5, 1.0, ["bottom", "top"],
                                              omega_transform=LogScalars() if log_w else None,
                                              **kw)
        out.update(_mesh_arrays(prefix, mesh, geom))
        out[prefix + "wall_distance"] = np.asarray(turb.wall_distance)
        out[prefix + "wall_distance_gradient"] = np.asarray(turb.wall_distance_gradient)
        out[prefix + "inlet"] = np.array([k_in, omega_in])
        n = mesh.n_cells
        states = _rans_states(rng, n, 2, k_in, omega_in, 2)
        if log_w:
            for x in states:
                x[4 * n:] = np.log(x[4 * n:])
        out[prefix + "states"] = np.stack(states)
        out[prefix + "residuals"] = np.stack([np.asarray(coupled.residual(jnp.asarray(x)))
                                              for x in states])
        v = rng.standard_normal(5 * n)
        scale = np.abs(states[0]) + 1e-3
        out[prefix + "jvp_dir"] = v * scale
        out[prefix + "jvp_fd"] = _fd_jvp(coupled.residual, states[0], v * scale, 1e-7)
    return out


# --------------------------------------------------------------------------- corrected gradients
def _swept(sweeps, relaxation=1.0):
    """CorrectedGreenGauss with a fixed sweep count (``aquaflux/schemes/gradient.py:547-705,
    1122-1337``); the convergence diagnostic is off (it only warns)."""
    return CorrectedGreenGauss(solver=SweptGradientSolve(sweeps=sweeps, warn_tol=None,
                                                         relaxation=relaxation))


def corrected_cases():
    out = {}
    rng = np.random.default_rng(31)
    # the standalone scheme on a jittered 2D mesh: a linear field (exact at convergence) and a
    # random field with random boundary values, at 4 and 24 sweeps
    m = structured_grid_2d(9, 7, lx=1.5, ly=1.0, named_boundaries=True)
    m = _with_nodes(m, jitter_interior_nodes(np.asarray(m.node_coords), (9, 7), (1.5, 1.0),
                                             0.2, 6))
    geom = m.geometry()
    out.update(_mesh_arrays("g2_", m, geom))
    cc = np.asarray(geom.cell.centroid)
    xf = np.asarray(geom.face.centroid)
    lin = 0.7 + 1.3 * cc[:, 0] - 2.1 * cc[:, 1]
    lin_b = 0.7 + 1.3 * xf[:, 0] - 2.1 * xf[:, 1]
    phi = rng.standard_normal(m.n_cells)
    phi_b = rng.standard_normal(len(xf))
    out["g2_fields"] = np.stack([lin, phi])
    out["g2_bvals"] = np.stack([lin_b, phi_b])
    for sw, rel in ((4, 1.0), (24, 1.0), (6, 0.8)):
        sch = _swept(sw, rel)
        out[f"g2_grad_s{sw}"] = np.stack([
            np.asarray(sch.gradients(jnp.asarray(f), m, geom, jnp.asarray(b)))
            for f, b in zip(out["g2_fields"], out["g2_bvals"])])
    # jittered cavity, 4 sweeps
    mesh, geom, asm = _cavity(10, perturb=0.15, seed=0, scheme=_swept(4))
    out.update(_mesh_arrays("ccavj_", mesh, geom))
    states = [rng.standard_normal(300) * 0.3, rng.standard_normal(300)]
    out["ccavj_states"] = np.stack(states)
    out["ccavj_residuals"] = np.stack([np.asarray(asm.residual(jnp.asarray(s))) for s in states])
    out.update(_flow_fields("ccavj_s0_", asm, states[0]))
    v = rng.standard_normal(300)
    out["ccavj_jvp_dir"] = v
    out["ccavj_jvp_fd"] = _fd_jvp(asm.residual, states[0], v, 1e-6)
    # 2D graded jittered SST channel, 4 sweeps (the corrected form of the backward-step physics)
    nx, ny = 12, 8
    yn = graded_nodes(ny, 1.0, 1.2)
    mesh = structured_grid_2d(nx, ny, lx=4.0, ly=1.0, named_boundaries=True, y_nodes=yn)
    mesh = _with_nodes(mesh, jitter_interior_nodes(np.asarray(mesh.node_coords), (nx, ny),
                                                   (4.0, 1.0), 0.15, 4))
    geom = mesh.geometry()
    coupled, turb, k_in, omega_in = _rans(mesh, geom, 2, 2e-5, 1.0, ["bottom", "top"],
                                          scheme=_swept(4))
    out.update(_mesh_arrays("csst2_", mesh, geom))
    out["csst2_y_nodes"] = np.asarray(yn)
    out["csst2_wall_distance"] = np.asarray(turb.wall_distance)
    out["csst2_wall_distance_gradient"] = np.asarray(turb.wall_distance_gradient)
    out["csst2_inlet"] = np.array([k_in, omega_in])
    n = mesh.n_cells
    states = _rans_states(rng, n, 2, k_in, omega_in, 2, negative_k=True)
    out["csst2_states"] = np.stack(states)
    out["csst2_residuals"] = np.stack([np.asarray(coupled.residual(jnp.asarray(s)))
                                       for s in states])
    v = rng.standard_normal(5 * n)
    scale = np.abs(states[0]) + 1e-3
    out["csst2_jvp_dir"] = v * scale
    out["csst2_jvp_fd"] = _fd_jvp(coupled.residual, states[0], v * scale, 1e-7)
    # 3D duct with a bump, 3 under-relaxed sweeps
    shape = (5, 4, 3)
    mesh = structured_grid_3d(*shape, lx=2.0, ly=1.0, lz=1.0, named_boundaries=True)
    mesh = _with_nodes(mesh, bump_channel_nodes_3d(shape, (2.0, 1.0, 1.0), 0.1, 0.1, 9))
    geom = mesh.geometry()
    walls = ["bottom", "top", "back", "front"]
    coupled, turb, k_in, omega_in = _rans(mesh, geom, 3, 1e-3, 1.0, walls,
                                          scheme=_swept(3, 0.8))
    out.update(_mesh_arrays("csst3_", mesh, geom))
    out["csst3_wall_distance"] = np.asarray(turb.wall_distance)
    out["csst3_wall_distance_gradient"] = np.asarray(turb.wall_distance_gradient)
    out["csst3_inlet"] = np.array([k_in, omega_in])
    n = mesh.n_cells
    states = _rans_states(rng, n, 3, k_in, omega_in, 2)
    out["csst3_states"] = np.stack(states)
    out["csst3_residuals"] = np.stack([np.asarray(coupled.residual(jnp.asarray(s)))
                                       for s in states])
    return out


# --------------------------------------------------------------------------- limited advection
def limited_cases():
    """``LimitedUpwind`` (``aquaflux/discretization/advection.py:117-157``) with the
    ``VenkatakrishnanLimiter`` (``aquaflux/schemes/limiter.py:78-117``, K = 5) and unlimited."""
    out = {}
    rng = np.random.default_rng(47)
    for prefix, adv in (("lcavj_", LimitedUpwind(limiter=VenkatakrishnanLimiter(k=5.0))),
                        ("ucavj_", LimitedUpwind(limiter=None))):
        mesh, geom, asm = _cavity(10, perturb=0.15, seed=0, advection=adv)
        out.update(_mesh_arrays(prefix, mesh, geom))
        states = [rng.standard_normal(300) * 0.3, rng.standard_normal(300)]
        out[prefix + "states"] = np.stack(states)
        out[prefix + "residuals"] = np.stack([np.asarray(asm.residual(jnp.asarray(x)))
                                              for x in states])
        v = rng.standard_normal(300)
        out[prefix + "jvp_dir"] = v
        out[prefix + "jvp_fd"] = _fd_jvp(asm.residual, states[0], v, 1e-6)
    nx, ny = 12, 8
    yn = graded_nodes(ny, 1.0, 1.2)
    mesh = structured_grid_2d(nx, ny, lx=4.0, ly=1.0, named_boundaries=True, y_nodes=yn)
    mesh = _with_nodes(mesh, jitter_interior_nodes(np.asarray(mesh.node_coords), (nx, ny),
                                                   (4.0, 1.0), 0.1, 4))
    geom = mesh.geometry()
    coupled, turb, k_in, omega_in = _rans(mesh, geom, 2, 2e-5, 1.0, ["bottom", "top"],
                                          advection=LimitedUpwind(
                                              limiter=VenkatakrishnanLimiter(k=5.0)))
    out.update(_mesh_arrays("lsst2_", mesh, geom))
    out["lsst2_inlet"] = np.array([k_in, omega_in])
    n = mesh.n_cells
    states = _rans_states(rng, n, 2, k_in, omega_in, 2)
    out["lsst2_states"] = np.stack(states)
    out["lsst2_residuals"] = np.stack([np.asarray(coupled.residual(jnp.asarray(x)))
                                       for x in states])
    v = rng.standard_normal(5 * n)
    scale = np.abs(states[0]) + 1e-3
    out["lsst2_jvp_dir"] = v * scale
    out["lsst2_jvp_fd"] = _fd_jvp(coupled.residual, states[0], v * scale, 1e-7)
    return out


# --------------------------------------------------------------------------- shifted operators
def operator_cases():
    """``ShiftedCellMajorOperator.assemble`` (``aquaflux/solve/amg_preconditioner.py:545-658``),
    ``shifted_jacobian`` (``sparse_jacobian.py:893-927``) and ``equilibrate_cell_major``
    (``frozen_operator.py:382-435``) on a block-stencil matrix in the field-major layout."""
    import scipy.sparse as sp

    from aquaflux.solve.amg_preconditioner import ShiftedCellMajorOperator
    from aquaflux.solve.frozen_operator import equilibrate_cell_major
    from aquaflux.solve.sparse_jacobian import shifted_jacobian

    out = {}
    rng = np.random.default_rng(41)
    mesh = structured_grid_2d(7, 5, named_boundaries=True)
    n, b = mesh.n_cells, 3
    own = np.asarray(mesh.face_cells.owner)
    nb = np.asarray(mesh.face_cells.neighbour)
    inner = nb >= 0
    rows = np.concatenate([own[inner], nb[inner], np.arange(n)])
    cols = np.concatenate([nb[inner], own[inner], np.arange(n)])
    pat = sp.csr_matrix((np.ones(rows.size), (rows, cols)), shape=(n, n))
    pat.sort_indices()
    nnzb = pat.nnz
    blocks = rng.standard_normal((nnzb, b, b))
    blocks[rng.random((nnzb, b, b)) < 0.1] = 0.0  # explicit zeros stay in the pattern
    dq = pat.indptr[:-1] + np.array([np.searchsorted(pat.indices[pat.indptr[i]:pat.indptr[i + 1]], i)
                                     for i in range(n)])
    blocks[dq, 2, 2] = 0.0  # zero pressure diagonal: the scale treats |0| as 1
    # field-major CSR with every block entry stored
    brow = np.repeat(np.arange(n), np.diff(pat.indptr))
    r = (np.arange(b)[None, :, None] * n + brow[:, None, None]) * np.ones((1, 1, b), dtype=np.int64)
    c = (np.arange(b)[None, None, :] * n + pat.indices[:, None, None]) * np.ones((1, b, 1), dtype=np.int64)
    coo = sp.coo_matrix((np.ones(r.size), (r.ravel(), c.ravel())), shape=(n * b, n * b)).tocsr()
    coo.sort_indices()
    # place the values into the sorted field-major pattern
    key = r.ravel() * (n * b) + c.ravel()
    order = np.argsort(key)
    fm_values = blocks.ravel()[order]
    shift = np.concatenate([rng.random(n) * 2.0, rng.random(n) * 2.0, np.zeros(n)])
    op = ShiftedCellMajorOperator(coo.indptr, coo.indices, b)
    mat, scale, perm = op.assemble(fm_values, shift)
    out["op_bsr_indptr"] = pat.indptr.astype(np.int32)
    out["op_bsr_indices"] = pat.indices.astype(np.int32)
    out["op_blocks"] = blocks
    out["op_shift"] = shift
    out["op_cm_indptr"] = np.asarray(mat.indptr)
    out["op_cm_indices"] = np.asarray(mat.indices)
    out["op_cm_data"] = np.asarray(mat.data).copy()
    out["op_scale"] = np.asarray(scale)
    out["op_perm"] = np.asarray(perm)
    fm = sp.csr_matrix((fm_values, coo.indices, coo.indptr), shape=coo.shape)
    out["op_shifted_fm_data"] = np.asarray(shifted_jacobian(fm, shift).data)
    eq, eq_scale, _ = equilibrate_cell_major(fm, b)
    out["op_eq_cm_data"] = np.asarray(eq.data)
    out["op_eq_scale"] = np.asarray(eq_scale)
    return out


# --------------------------------------------------------------------------- ILU(0)
def ilu_cases():
    import test_ilu0  # the reference's own unit test module (its fixture operator)

    a = test_ilu0._nonsymmetric()
    a.sort_indices()
    n = a.shape[0]
    indptr = a.indptr.astype(np.int32)
    indices = a.indices.astype(np.int32)
    diag = ref_ilu0._diagonal_positions(indptr, indices, n)
    data = a.data.astype(np.float64).copy()
    ref_ilu0._reference_factor(indptr, indices, data, diag, n)
    rng = np.random.default_rng(31)
    rhs = rng.standard_normal(n)
    x = rhs.copy()
    ref_ilu0._reference_solve(indptr, indices, data, diag, x, n)
    xt = rhs.copy()
    ref_ilu0._reference_solve_transpose(indptr, indices, data, diag, xt, n)
    return {"ilu_indptr": indptr, "ilu_indices": indices, "ilu_values": a.data.astype(np.float64),
            "ilu_diag": diag.astype(np.int32), "ilu_factor": data, "ilu_rhs": rhs,
            "ilu_solve": x, "ilu_solve_t": xt}


# --------------------------------------------------------------------------- colouring
def colouring_cases():
    """``block_stencil_colouring`` (``aquaflux/solve/sparse_jacobian.py:338-402``) on the interior
    face graphs of small 2D / 3D meshes (one relabelled at random), reaches 1-3."""
    from aquaflux.mesh import RandomReordering, permute_cells
    from aquaflux.solve.sparse_jacobian import block_stencil_colouring

    out = {}
    meshes = {"c2d": structured_grid_2d(9, 7, named_boundaries=True),
              "c3d": structured_grid_3d(5, 4, 3, named_boundaries=True)}
    m = structured_grid_3d(4, 4, 3, named_boundaries=True)
    meshes["c3p"] = permute_cells(m, RandomReordering(seed=3).permutation(m))
    for name, mesh in meshes.items():
        o, nb, _ = mesh.face_cells.interior_edges()
        out[f"{name}_owner"] = o.astype(np.int32)
        out[f"{name}_nb"] = nb.astype(np.int32)
        out[f"{name}_n"] = np.array(mesh.n_cells)
        for reach in (1, 2, 3):
            col = block_stencil_colouring(o, nb, mesh.n_cells, reach)
            out[f"{name}_r{reach}_colour"] = np.asarray(col.colour).astype(np.int32)
            out[f"{name}_r{reach}_rows"] = np.asarray(col.pattern_rows).astype(np.int32)
            out[f"{name}_r{reach}_cols"] = np.asarray(col.pattern_cols).astype(np.int32)
    return out


# polyMesh directories read by the reference's importer: its own unit-test fixtures and the
# validation cases that ship a mesh (paths relative to the reference checkout).
POLYMESH_DIRS = {
    "slab2d": "tests/fixtures/polymesh_2d_slab",
    "slab2d_fb": "tests/fixtures/polymesh_2d_slab_frontandback",
    "cubes3d": "tests/fixtures/polymesh_3d_two_cubes",
    "pitzdaily": "validation/pitzdaily_openfoam/of_case",
    "bfs3d": "validation/bfs3d_species/of_case",
}


def _digest(a, dtype):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(np.asarray(a), dtype=dtype).tobytes()).hexdigest()


def openfoam_cases():
    """``read_openfoam`` (``aquaflux/io/openfoam/reader.py:133``) on the reference's polyMesh
    directories.  The meshes themselves stay in the reference checkout: only SHA-256 digests of the
    imported arrays (node coordinates as float64, connectivity as int64, each patch's face indices)
    and the geometry totals are kept, so the import tests compare against them wherever the
    reference checkout is present."""
    from aquaflux.io import read_openfoam
    out = {}
    for key, rel in POLYMESH_DIRS.items():
        m = read_openfoam(os.path.join(REF, rel))
        fc, fn = m.face_cells, m.face_nodes
        geom = m.geometry()
        out[f"{key}_counts"] = np.array([m.dim, m.n_cells, m.n_faces,
                                         np.asarray(m.node_coords).shape[0]], dtype=np.int64)
        out[f"{key}_digest"] = np.array([
            _digest(m.node_coords, np.float64), _digest(fn.offsets, np.int64),
            _digest(fn.face_node_indices, np.int64), _digest(fc.owner, np.int64),
            _digest(fc.neighbour, np.int64)])
        names = [n for n in m.face_patches.names if n not in ("interior", "boundary")]
        out[f"{key}_patch_names"] = np.array(names)
        out[f"{key}_patch_digest"] = np.array(
            [_digest(m.face_patches.indices(n), np.int64) for n in names])
        vol = np.asarray(geom.cell.volume)
        out[f"{key}_geometry"] = np.array([vol.sum(), np.abs(np.asarray(geom.face.area)).sum(),
                                           *(vol[:, None] * np.asarray(geom.cell.centroid)).sum(0)])
    return out


FILES = {"colouring": lambda: colouring_cases(), "meshes": lambda: mesh_cases(),
         "laminar": lambda: laminar_cases(), "sst": lambda: sst_cases(),
         "ilu0": lambda: ilu_cases(), "corrected": lambda: corrected_cases(),
         "operator": lambda: operator_cases(), "limited": lambda: limited_cases(),
         "openfoam": lambda: openfoam_cases(), "logscalars": lambda: logscalar_cases(),
         "mixed": lambda: mixed_cases()}


def main():
    """``make_golden.py REF [name ...]``: regenerate the named fixture files (default: all)."""
    names = sys.argv[2:] or list(FILES)
    for f in names:
        np.savez_compressed(os.path.join(HERE, f + ".npz"), **FILES[f]())
        print(f, os.path.getsize(os.path.join(HERE, f + ".npz")))


if __name__ == "__main__":
    main()
