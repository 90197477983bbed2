"""CPU oracle for the finite-volume hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import this
module, and only as the checker.  The product (``aquaflux_gb300``) never calls it.

It restates, in float64 torch on the CPU, the reference's forward path:

* face/cell geometry (``aquaflux/mesh/face.py:217-349``, ``aquaflux/mesh/cell.py:84-170``,
  ``aquaflux/mesh/mesh.py:366-387``);
* the coupled momentum + Rhie-Chow continuity residual with compact Green-Gauss gradients and
  first-order upwind advection (``aquaflux/flow/momentum.py:233-882``,
  ``aquaflux/flow/rhie_chow.py:81-353``, ``aquaflux/flow/boundary.py:43-446``,
  ``aquaflux/discretization/diffusion.py:59-199``, ``aquaflux/discretization/advection.py:41-187``,
  ``aquaflux/schemes/gradient.py:129-153``, ``aquaflux/schemes/interpolation.py:27-176``);
* the k-omega SST closure and the coupled RANS residual (``aquaflux/turbulence/sst.py:37-239``,
  ``aquaflux/turbulence/sources.py:60-412``, ``aquaflux/turbulence/boundary.py:45-589``,
  ``aquaflux/turbulence/transport.py:369-718``, ``aquaflux/turbulence/coupled.py:437-473``).

Because it is written in torch, ``torch.func.jvp`` / ``torch.autograd`` of :func:`residual` give the
JVP / VJP oracle with respect to the state, the physical parameters and the node coordinates.

Its parity is pinned by ``tests/test_oracle_golden.py`` against golden vectors generated by the
reference package itself (``tests/golden/make_golden.py``).

Boundary conditions arrive as a flat per-face table (see :func:`make_case`):
``bc_kind``: -1 interior / unpatched, 0 no-slip wall, 1 moving wall, 2 velocity inlet,
3 pressure outlet; ``bc_vel`` (F, dim) prescribed velocity; ``bc_p`` (F,) outlet pressure.
Scalar (k, omega) boundary kinds: 0 Dirichlet (value in ``*_val``), 1 zero gradient.
"""
from __future__ import annotations

import math

import numpy as np
import torch

T = torch.float64

# SST constants, ``aquaflux/turbulence/sst.py:69-82``.
A1, BETA_STAR, ALPHA_1, BETA_1 = 0.31, 0.09, 5.0 / 9.0, 3.0 / 40.0
SIGMA_K1, SIGMA_W1, ALPHA_2, BETA_2 = 0.85, 0.5, 0.44, 0.0828
SIGMA_K2, SIGMA_W2, KAPPA, E_WALL = 1.0, 0.856, 0.41, 9.8
WALL_OMEGA_EXPONENT, WALL_OMEGA_VISCOUS = 2.0, 1.0
CROSS_DIFFUSION_FLOOR = 1e-10  # sst.py:34
PRODUCTION_LIMIT_RATIO = 10.0  # sources.py:52
EDDY_VISCOSITY_FLOOR = 1e-30  # sources.py:57


def wall_y_star_lam() -> float:
    """Ten fixed-point sweeps of ``y = ln(E y) / kappa`` from 11 (``sst.py:86-106``)."""
    y = 11.0
    for _ in range(10):
        y = math.log(E_WALL * y) / KAPPA
    return y


Y_LAM = wall_y_star_lam()


# ----------------------------------------------------------------------------- helpers
def _t(x, dtype=T):
    return torch.as_tensor(np.asarray(x), dtype=dtype)


def _dot(a, b):
    """Component sum left to right (``aquaflux/vectors.py:28-65``)."""
    p = a * b
    out = p[..., 0]
    for i in range(1, p.shape[-1]):
        out = out + p[..., i]
    return out


def _segsum(values, index, n):
    out = torch.zeros((n,) + tuple(values.shape[1:]), dtype=values.dtype)
    return out.index_add(0, index, values)


class Topology:
    """Face->cell and face->node incidence as torch index tensors."""

    def __init__(self, owner, neighbour, n_cells, fn_offsets, fn_indices):
        self.owner = _t(owner, torch.long)
        self.neighbour = _t(neighbour, torch.long)
        self.n_cells = int(n_cells)
        self.n_faces = int(self.owner.shape[0])
        self.interior = self.neighbour >= 0
        self.safe_nb = torch.where(self.interior, self.neighbour, self.owner)
        self.nb_scatter = torch.where(self.interior, self.neighbour,
                                      torch.full_like(self.neighbour, self.n_cells))
        off = np.asarray(fn_offsets, dtype=np.int64)
        idx = np.asarray(fn_indices, dtype=np.int64)
        counts = np.diff(off)
        inc_face = np.repeat(np.arange(self.n_faces), counts)
        starts = off[:-1][inc_face]
        local = np.arange(idx.size) - starts
        nxt = starts + (local + 1) % counts[inc_face]
        self.fn_indices = torch.as_tensor(idx)
        self.inc_face = torch.as_tensor(inc_face)
        self.next_inc = torch.as_tensor(nxt)
        self.counts = torch.as_tensor(counts, dtype=T)

    def scatter(self, own, nb):
        """``FaceCellConnectivity.scatter`` (``aquaflux/mesh/connectivity.py:236-260``)."""
        a = _segsum(own, self.owner, self.n_cells)
        b = _segsum(nb, self.nb_scatter, self.n_cells + 1)[: self.n_cells]
        return a + b

    def scatter_conservative(self, flux):
        return self.scatter(flux, -flux)

    def blend(self, own_field, nb_field, g):
        gg = g.reshape(g.shape + (1,) * (own_field.dim() - 1))
        return (1.0 - gg) * own_field[self.owner] + gg * nb_field[self.safe_nb]

    def combine(self, interior_values, boundary_values):
        mask = self.interior.reshape(self.interior.shape + (1,) * (interior_values.dim() - 1))
        return torch.where(mask, interior_values, boundary_values)


def _safe_norm(v):
    sq = _dot(v, v)
    pos = sq > 0.0
    return torch.where(pos, torch.sqrt(torch.where(pos, sq, torch.ones_like(sq))),
                       torch.zeros_like(sq))


def _safe_unit(v):
    sq = torch.sum(v * v, dim=-1, keepdim=True)
    pos = sq > 0.0
    return torch.where(pos, v / torch.sqrt(torch.where(pos, sq, torch.ones_like(sq))),
                       torch.zeros_like(v))


# ----------------------------------------------------------------------------- geometry
def geometry(topo: Topology, nodes: torch.Tensor) -> dict:
    """Face area / centroid / owner-outward normal, cell volume / centroid.

    ``Mesh.geometry`` -> ``_fused_geometry`` (``aquaflux/mesh/mesh.py:366-387``): edge or centre-fan
    face geometry (``face.py:217-230, 292-349``), face-centroid-mean approximate cell centroids
    (``cell.py:84-108``), owner-outward flip (``face.py:196-211``), recentred divergence-theorem
    volume and centroid (``cell.py:124-170``).
    """
    dim = nodes.shape[1]
    nf = topo.n_faces
    if dim == 2:
        verts = nodes[topo.fn_indices].reshape(nf, 2, 2)
        p0, p1 = verts[:, 0], verts[:, 1]
        d = p1 - p0
        area = _safe_norm(d)
        centroid = 0.5 * (p0 + p1)
        normal = _safe_unit(torch.stack([d[:, 1], -d[:, 0]], dim=1))
    else:
        pb = nodes[topo.fn_indices]
        pc = pb[topo.next_inc]
        vmean = _segsum(pb, topo.inc_face, nf) * (1.0 / topo.counts)[:, None]
        pa = vmean[topo.inc_face]
        directed = 0.5 * torch.linalg.cross(pb - pa, pc - pa, dim=-1)
        tri_c = (pa + pb + pc) / 3.0
        s = _segsum(directed, topo.inc_face, nf)
        area = _safe_norm(s)
        normal = _safe_unit(s)
        signed = _dot(directed, normal[topo.inc_face])
        safe_area = torch.where(area > 0.0, area, torch.ones_like(area))[:, None]
        centroid = _segsum(signed[:, None] * tri_c, topo.inc_face, nf) / safe_area
    ones = torch.ones(nf, dtype=T)
    count = topo.scatter(ones, ones)
    approx = topo.scatter(centroid, centroid) * (1.0 / count)[:, None]
    outward = centroid - approx[topo.owner]
    proj = torch.sum(outward * normal, dim=1, keepdim=True)
    normal = normal * torch.where(proj < 0.0, -1.0, 1.0)
    own_local = centroid - approx[topo.owner]
    nb_local = centroid - approx[topo.safe_nb]
    flux = _dot(own_local, normal) * area
    nflux = _dot(nb_local, normal) * area
    volume = topo.scatter(flux, -nflux) / dim
    csum = topo.scatter(flux[:, None] * own_local, -(nflux[:, None] * nb_local))
    cell_centroid = csum * (1.0 / ((dim + 1) * volume))[:, None] + approx
    return {"area": area, "normal": normal, "face_centroid": centroid, "volume": volume,
            "cell_centroid": cell_centroid}


class Metrics:
    """Geometry-derived per-face factors (``MomentumContinuity.build``, ``momentum.py:233-293``)."""

    def __init__(self, topo: Topology, geo: dict):
        self.topo, self.geo = topo, geo
        cc, xf, n = geo["cell_centroid"], geo["face_centroid"], geo["normal"]
        x_p = cc[topo.owner]
        d = cc[topo.safe_nb] - x_p
        dd = torch.where(topo.interior, _dot(d, d), torch.ones_like(d[:, 0]))
        self.g = torch.where(topo.interior, _dot(xf - x_p, d) / dd, torch.zeros_like(dd))
        self.d = d
        self.normal_distance = torch.where(topo.interior, _dot(d, n), _dot(xf - x_p, n))
        self.skew = xf - (x_p + d * self.g[:, None])
        self.d_p = xf - x_p
        self.d_n = xf - cc[topo.safe_nb]
        self.dpn = _dot(self.d_p, n)
        self.dnn = _dot(self.d_n, n)
        self.area_vector = n * geo["area"][:, None]


def gg_gradient(m: Metrics, phi, bvals, scheme=None):
    """Compact Green-Gauss, ``aquaflux/schemes/gradient.py:129-153``; with ``scheme =
    {"sweeps": s, "relaxation": r}`` the corrected Green-Gauss reconstruction of
    ``CorrectedGreenGauss`` (``gradient.py:1122-1337``: operator ``A_g G = V G - C(G)`` with the
    skewness coupling ``C``, right-hand side ``B phi`` = the compact numerator) solved by
    ``SweptGradientSolve`` (``gradient.py:618-705``: the peeled first sweep ``x = r P^-1 B phi``,
    then ``s - 1`` sweeps ``x += r P^-1 (B phi - A_g x)``, ``P^-1 = 1 / V``)."""
    topo = m.topo
    phi_face = topo.combine(topo.blend(phi, phi, m.g), bvals)
    gsum = topo.scatter_conservative(m.area_vector * phi_face[:, None])
    inv_v = (1.0 / m.geo["volume"])[:, None]
    if scheme is None or scheme["sweeps"] <= 1 and scheme.get("relaxation", 1.0) == 1.0:
        return gsum * inv_v
    rel = scheme.get("relaxation", 1.0)
    vol = m.geo["volume"][:, None]
    x = rel * (gsum * inv_v)
    o, nb = topo.owner, topo.safe_nb
    for _ in range(scheme["sweeps"] - 1):
        w = (1.0 - m.g) * _dot(m.skew, x[o]) + m.g * _dot(m.skew, x[nb])
        face = torch.where(topo.interior[:, None], m.area_vector * w[:, None],
                           torch.zeros_like(m.area_vector))
        ax = x * vol - topo.scatter_conservative(face)
        x = x + rel * ((gsum - ax) * inv_v)
    return x


def interpolate_to_face(m: Metrics, field, grad):
    """Skew-corrected face value, ``aquaflux/schemes/interpolation.py:125-176``."""
    topo = m.topo
    blend = topo.blend(field, field, m.g)
    grad_face = topo.blend(grad, grad, m.g)
    return blend + torch.einsum("f...j,fj->f...", grad_face, m.skew)


def _tangential(grad_owner, d, n):
    return _dot(grad_owner, d - n * _dot(d, n)[:, None])


def diffusion_flux(m: Metrics, phi, grad, gamma, bvals, boundary_coefficient=None):
    """``DiffusionFlux.face_flux``, ``aquaflux/discretization/diffusion.py:163-199``."""
    topo, n, area = m.topo, m.geo["normal"], m.geo["area"]
    o, nb = topo.owner, topo.safe_nb
    corr_p = _dot(grad[o], m.d_p - n * m.dpn[:, None])
    corr_n = _dot(grad[nb], m.d_n - n * m.dnn[:, None])
    denom = m.dpn - gamma[o] / gamma[nb] * m.dnn
    denom_safe = torch.where(topo.interior, denom, torch.ones_like(denom))
    ng_i = (phi[nb] - phi[o] + corr_n - corr_p) / denom_safe
    ng_b = (bvals - phi[o] - corr_p) / m.dpn
    ng = torch.where(topo.interior, ng_i, ng_b)
    gamma_face = gamma[o]
    if boundary_coefficient is not None:
        gamma_face = torch.where(topo.interior, gamma_face, boundary_coefficient)
    return -gamma_face * ng * area


def upwind_flux(m: Metrics, phi, mass_flux, bvals):
    """``FirstOrderUpwind`` + ``AdvectionFlux`` (``aquaflux/discretization/advection.py:99-187``)."""
    topo = m.topo
    out = mass_flux >= 0.0
    interior_value = torch.where(out, phi[topo.owner], phi[topo.safe_nb])
    boundary_value = torch.where(out, phi[topo.owner], bvals)
    return mass_flux * torch.where(topo.interior, interior_value, boundary_value)


def venkatakrishnan(m: Metrics, phi, grad, k):
    """``VenkatakrishnanLimiter.limit`` (``aquaflux/schemes/limiter.py:78-117``): per-cell
    ``psi = clip(min over faces of psi_face, 0, 1)`` with the stencil extrema over the interior
    neighbours and ``eps^2 = V K^3``."""
    topo = m.topo
    o, nb, inter = topo.owner, topo.safe_nb, topo.interior
    geo = m.geo
    nc = topo.n_cells
    io, inb = o[inter], nb[inter]
    idx = torch.cat([io, inb])
    src = torch.cat([phi[inb], phi[io]])
    pmax = phi.scatter_reduce(0, idx, src, reduce="amax", include_self=True)
    pmin = phi.scatter_reduce(0, idx, src, reduce="amin", include_self=True)
    eps2 = geo["volume"] * k ** 3
    xf, xc = geo["face_centroid"], geo["cell_centroid"]

    def face_limiter(cell):
        dm = _dot(grad[cell], xf - xc[cell])
        sign = torch.where(dm >= 0.0, torch.ones_like(dm), -torch.ones_like(dm))
        dm = sign * (torch.abs(dm) + 1e-12)
        head = torch.where(dm > 0.0, pmax[cell] - phi[cell], pmin[cell] - phi[cell])
        e2 = eps2[cell]
        num = (head ** 2 + e2) * dm + 2.0 * dm ** 2 * head
        den = (head ** 2 + 2.0 * dm ** 2 + head * dm + e2) * dm
        return num / den

    lo, ln = face_limiter(o), face_limiter(nb)
    big = torch.full((nc,), float("inf"), dtype=T)
    psi = big.scatter_reduce(0, torch.cat([o, inb]), torch.cat([lo, ln[inter]]), reduce="amin",
                             include_self=True)
    return torch.clamp(psi, 0.0, 1.0)


def advected_face_value(m: Metrics, phi, grad, mass_flux, bvals, scheme):
    """The advected face value: ``FirstOrderUpwind`` (``scheme`` None) or ``LimitedUpwind``
    (``aquaflux/discretization/advection.py:117-157``: ``phi_C + psi_C grad phi_C . (x_f - x_C)``
    from the upwind cell, ``psi`` Venkatakrishnan with ``K = scheme["k"]`` or 1 when ``k`` is
    None); boundary inflow takes the weak boundary value."""
    topo = m.topo
    out = mass_flux >= 0.0
    if scheme is None:
        interior_value = torch.where(out, phi[topo.owner], phi[topo.safe_nb])
        boundary_value = torch.where(out, phi[topo.owner], bvals)
        return torch.where(topo.interior, interior_value, boundary_value)
    psi = (torch.ones_like(phi) if scheme.get("k") is None
           else venkatakrishnan(m, phi, grad, scheme["k"]))
    o, nb = topo.owner, topo.safe_nb
    xc, xf = m.geo["cell_centroid"], m.geo["face_centroid"]
    phi_up = torch.where(out, phi[o], phi[nb])
    psi_up = torch.where(out, psi[o], psi[nb])
    grad_up = torch.where(out[:, None], grad[o], grad[nb])
    x_up = torch.where(out[:, None], xc[o], xc[nb])
    rec = phi_up + psi_up * _dot(grad_up, xf - x_up)
    return torch.where(topo.interior | out, rec, bvals)


def advection_flux(m: Metrics, phi, grad, mass_flux, bvals, scheme):
    """``AdvectionFlux.face_flux``: ``mdot_f phi_f``."""
    return mass_flux * advected_face_value(m, phi, grad, mass_flux, bvals, scheme)


# ----------------------------------------------------------------------------- the case
def make_case(mesh, *, mu, rho, flow_bc, pressure_pin=None, pressure_pin_value=0.0, sst=None,
              gradient=None, advection=None, transforms=("direct", "direct"),
              scalar_advection=None):
    """Flatten a case description into per-face tables.

    ``mesh``: object with ``nodes, fn_offsets, fn_indices, owner, neighbour, n_cells, patches``.
    ``flow_bc``: ``{patch: ("wall",) | ("moving", U) | ("inlet", U) | ("outlet", p)}``.
    ``sst``: ``None`` or ``{"nu": float, "walls": [patches], "k": {patch: ("dirichlet", v) |
    ("zerograd",)}, "omega": {...}}``.
    ``gradient``: ``None`` (compact Green-Gauss) or ``{"sweeps": s, "relaxation": r}`` (corrected
    Green-Gauss by ``s`` swept sweeps).
    ``advection``: ``None`` (first-order upwind) or ``{"k": K}`` (limited linear upwind with the
    Venkatakrishnan limiter, ``K`` None for the unlimited reconstruction).
    ``transforms``: the solved variables of k and omega, ``"direct"`` or ``"log"`` (``DirectScalars``
    / ``LogScalars``, ``aquaflux/turbulence/coupled.py:111-207``).
    ``scalar_advection``: the k / omega advection scheme when it is not the momentum's (the
    reference builds ``SSTTurbulence`` with its own scheme): ``"upwind"`` or a dict like
    ``advection``.
    """
    nf = len(mesh.owner)
    dim = mesh.nodes.shape[1]
    kind = np.full(nf, -1, dtype=np.int64)
    vel = np.zeros((nf, dim))
    pb = np.zeros(nf)
    codes = {"wall": 0, "moving": 1, "inlet": 2, "outlet": 3}
    for name, spec in flow_bc.items():
        faces = np.asarray(mesh.patches[name], dtype=np.int64)
        kind[faces] = codes[spec[0]]
        if spec[0] in ("moving", "inlet"):
            vel[faces] = np.asarray(spec[1], dtype=float)
        if spec[0] == "outlet":
            pb[faces] = float(spec[1])
    case = {"mesh": mesh, "dim": dim, "mu": float(mu), "rho": float(rho), "bc_kind": kind,
            "bc_vel": vel, "bc_p": pb, "pin": pressure_pin, "pin_value": float(pressure_pin_value),
            "sst": None, "gradient": gradient, "advection": advection,
            "transforms": tuple(transforms),
            "scalar_advection": advection if scalar_advection is None else
            (None if scalar_advection == "upwind" else scalar_advection)}
    if sst is not None:
        sc = {"nu": float(sst["nu"])}
        for fld in ("k", "omega"):
            kk = np.full(nf, -1, dtype=np.int64)
            vv = np.zeros(nf)
            for name, spec in sst[fld].items():
                faces = np.asarray(mesh.patches[name], dtype=np.int64)
                kk[faces] = 0 if spec[0] == "dirichlet" else 1
                if spec[0] == "dirichlet":
                    vv[faces] = float(spec[1])
            sc[fld + "_kind"], sc[fld + "_val"] = kk, vv
        wall_faces = np.concatenate([np.asarray(mesh.patches[p], dtype=np.int64)
                                     for p in sst["walls"]])
        sc["wall_faces"] = wall_faces
        sc["wall_cells"] = np.unique(np.asarray(mesh.owner)[wall_faces]).astype(np.int64)
        case["sst"] = sc
    return case


def wall_distance(case, geo) -> tuple[torch.Tensor, torch.Tensor]:
    """Nearest wall-face-centroid distance and its Green-Gauss gradient.

    ``distance_to_patches`` (``aquaflux/mesh/distance.py:52-84``, exact nearest neighbour) and
    ``_reconstruct_wall_distance_gradient`` (``aquaflux/turbulence/transport.py:86-111``: Dirichlet 0
    on the walls, zero gradient elsewhere, one compact Green-Gauss pass).
    """
    sc = case["sst"]
    mesh = case["mesh"]
    topo = Topology(mesh.owner, mesh.neighbour, mesh.n_cells, mesh.fn_offsets, mesh.fn_indices)
    cc = geo["cell_centroid"].detach().numpy()
    tgt = geo["face_centroid"].detach().numpy()[sc["wall_faces"]]
    if cc.shape[0] * tgt.shape[0] <= 5e7:
        best = np.full(cc.shape[0], np.inf)
        for start in range(0, tgt.shape[0], 256):
            blk = tgt[start:start + 256]
            d2 = ((cc[:, None, :] - blk[None, :, :]) ** 2).sum(-1)
            best = np.minimum(best, d2.min(axis=1))
    else:  # large meshes: the nearest wall face by a k-d tree, the distance recomputed as above
        from scipy.spatial import cKDTree

        _, idx = cKDTree(tgt).query(cc, k=1)
        best = ((cc - tgt[idx]) ** 2).sum(-1)
    dist = torch.as_tensor(np.sqrt(best), dtype=T)
    m = Metrics(topo, {k: v.detach() for k, v in geo.items()})
    is_wall = np.zeros(topo.n_faces, dtype=bool)
    is_wall[sc["wall_faces"]] = True
    bvals = torch.where(torch.as_tensor(is_wall), torch.zeros(topo.n_faces, dtype=T),
                        dist[topo.owner])
    return dist, gg_gradient(m, dist, bvals, case.get("gradient"))


def nearest_wall_face(case, geo) -> np.ndarray:
    """Index (into the face arrays) of every cell's nearest SST wall-face centroid, first minimum."""
    sc = case["sst"]
    cc = geo["cell_centroid"].detach().numpy()
    wf = np.asarray(sc["wall_faces"])
    tgt = geo["face_centroid"].detach().numpy()[wf]
    best = np.full(cc.shape[0], np.inf)
    arg = np.zeros(cc.shape[0], dtype=np.int64)
    for start in range(0, tgt.shape[0], 256):
        blk = tgt[start:start + 256]
        d2 = ((cc[:, None, :] - blk[None, :, :]) ** 2).sum(-1)
        k = d2.argmin(axis=1)
        v = d2[np.arange(cc.shape[0]), k]
        better = v < best
        best = np.where(better, v, best)
        arg = np.where(better, start + k, arg)
    return wf[arg]


def wall_distance_live(case, geo, m, nearest):
    """The wall distance and its gradient as differentiable functions of the geometry, the nearest
    wall face held fixed (the mesh-coordinate derivative of ``distance_to_patches``)."""
    sc = case["sst"]
    topo = m.topo
    dv = geo["cell_centroid"] - geo["face_centroid"][torch.as_tensor(nearest)]
    dist = torch.sqrt((dv * dv).sum(-1))
    is_wall = np.zeros(topo.n_faces, dtype=bool)
    is_wall[sc["wall_faces"]] = True
    bvals = torch.where(torch.as_tensor(is_wall), torch.zeros(topo.n_faces, dtype=T),
                        dist[topo.owner])
    return dist, gg_gradient(m, dist, bvals, case.get("gradient"))


# ----------------------------------------------------------------------------- SST pieces
def safe_sqrt(x):
    pos = x > 0.0
    return torch.where(pos, torch.sqrt(torch.where(pos, x, torch.ones_like(x))), torch.zeros_like(x))


def wall_y_star(nu, d, k):
    return BETA_STAR ** 0.25 * safe_sqrt(torch.clamp(k, min=0.0)) * d / nu


def wall_function_weight(nu, d, k):
    return torch.tanh((wall_y_star(nu, d, k) / Y_LAM) ** 4)


def log_layer_shear_rate(d, k):
    return BETA_STAR ** 0.25 * safe_sqrt(torch.clamp(k, min=0.0)) / (KAPPA * d)


def _power_mean(a, b, p):
    m = torch.maximum(a, b)
    ra, rb = a / m, b / m
    pos = rb > 0.0
    rbs = torch.where(pos, rb, torch.ones_like(rb))
    bt = torch.where(pos, rbs ** p, torch.zeros_like(rb))
    return m * (ra ** p + bt) ** (1.0 / p)


def omega_wall(nu, d, k):
    """``aquaflux/turbulence/boundary.py:82-175``."""
    vis = WALL_OMEGA_VISCOUS * (6.0 * nu / (BETA_1 * d ** 2))
    log = safe_sqrt(torch.clamp(k, min=0.0)) / (BETA_STAR ** 0.25 * KAPPA * d)
    return _power_mean(vis, log, WALL_OMEGA_EXPONENT)


def nut_wall(nu, d, k):
    """``aquaflux/turbulence/boundary.py:177-231``."""
    ys = wall_y_star(nu, d, k)
    log_arg = E_WALL * torch.clamp(ys, min=Y_LAM)
    ratio = ys * KAPPA / torch.log(log_arg) - 1.0
    return nu * torch.where(ys > Y_LAM, ratio, torch.zeros_like(ratio))


def _omega_wall_gradient_live(nu, d, k, grad_d, grad_k):
    """Imposed wall-cell omega gradient, ``aquaflux/turbulence/boundary.py:535-589``.

    The reference takes ``d omega_wall / d d`` and ``d omega_wall / d k`` with ``jax.grad``; here
    the same derivatives are written in closed form (power mean with exponent 2, safe-sqrt
    subgradient 0 at k <= 0) so that torch can differentiate them again for the residual's JVP.
    """
    vis = WALL_OMEGA_VISCOUS * (6.0 * nu / (BETA_1 * d ** 2))
    kp = torch.clamp(k, min=0.0)
    sk = safe_sqrt(kp)
    c = BETA_STAR ** 0.25 * KAPPA
    log = sk / (c * d)
    dvis_dd = -2.0 * vis / d
    dlog_dd = -log / d
    # d sqrt(k)/dk with the safe-sqrt / clamp subgradient: 1/(2 sqrt k) for k > 0, else 0.
    pos = kp > 0.0
    dsk = torch.where(pos, 0.5 / torch.where(pos, sk, torch.ones_like(sk)), torch.zeros_like(sk))
    dlog_dk = dsk / (c * d)
    # omega = sqrt(vis^2 + log^2) (power mean, p = 2, written with the max-normalised form).
    w = _power_mean(vis, log, WALL_OMEGA_EXPONENT)
    dw_dvis = vis / w
    dw_dlog = log / w
    dwdd = dw_dvis * dvis_dd + dw_dlog * dlog_dd
    dwdk = dw_dlog * dlog_dk
    return grad_d * dwdd[:, None] + grad_k * dwdk[:, None]


def strain_rate_magnitude(grad_u):
    s = 0.5 * (grad_u + grad_u.transpose(-1, -2))
    return safe_sqrt(2.0 * torch.sum(s * s, dim=(-2, -1)))


def sst_f2(k, w, nu, d):
    arg2 = torch.maximum(2.0 * safe_sqrt(torch.clamp(k, min=0.0)) / (BETA_STAR * w * d),
                         500.0 * nu / (d ** 2 * w))
    return torch.tanh(arg2 ** 2)


def sst_f1(k, w, nu, d, gk, gw):
    cd = torch.clamp(2.0 * SIGMA_W2 * _dot(gk, gw) / w, min=CROSS_DIFFUSION_FLOOR)
    kp = torch.clamp(k, min=0.0)
    arg1 = torch.minimum(
        torch.maximum(safe_sqrt(kp) / (BETA_STAR * w * d), 500.0 * nu / (d ** 2 * w)),
        4.0 * SIGMA_W2 * kp / (cd * d ** 2))
    return torch.tanh(arg1 ** 4)


def sst_nut(k, w, strain, nu, d):
    return A1 * torch.clamp(k, min=0.0) / torch.maximum(A1 * w, strain * sst_f2(k, w, nu, d))


def blend(f1, inner, outer):
    return f1 * inner + (1.0 - f1) * outer


# ----------------------------------------------------------------------------- residual
class Oracle:
    """Residual oracle bound to one case.  ``residual(state)`` is differentiable in torch."""

    def __init__(self, case, nodes=None):
        self.case = case
        self._live_geometry = False
        mesh = case["mesh"]
        self.topo = Topology(mesh.owner, mesh.neighbour, mesh.n_cells, mesh.fn_offsets,
                             mesh.fn_indices)
        self.dim = case["dim"]
        self.nodes = _t(mesh.nodes) if nodes is None else nodes
        self.kind = torch.as_tensor(case["bc_kind"])
        self.bc_vel = _t(case["bc_vel"])
        self.bc_p = _t(case["bc_p"])
        if case["sst"] is not None:
            geo0 = geometry(self.topo, _t(mesh.nodes))
            self.wall_d, self.wall_dgrad = wall_distance(case, geo0)
            self._nearest = None

    # --- boundary tables ----------------------------------------------------------------------
    def _boundary_velocity(self, u):
        o = self.topo.owner
        k = self.kind[:, None]
        return torch.where(k == 3, u[o], torch.where((k == 1) | (k == 2), self.bc_vel,
                                                      torch.zeros_like(self.bc_vel)))

    def _boundary_pressure(self, p):
        o = self.topo.owner
        return torch.where(self.kind == 3, self.bc_p,
                           torch.where(self.kind >= 0, p[o], torch.zeros_like(p[o])))

    def _scalar_bvals(self, phi, grad, kind, val, geo):
        o = self.topo.owner
        kind = torch.as_tensor(kind)
        val = _t(val)
        if grad is None:
            zg = phi[o]
        else:
            d = geo["face_centroid"] - geo["cell_centroid"][o]
            zg = phi[o] + _tangential(grad[o], d, geo["normal"])
        return torch.where(kind == 0, val, torch.where(kind == 1, zg, torch.zeros_like(zg)))

    # --- the residual -------------------------------------------------------------------------
    def residual(self, state, *, mu=None, nodes=None, inlet_scale=None, return_fields=False):
        """``MomentumContinuity.residual`` / ``CoupledRANS.residual`` for this case.

        ``mu`` (molecular dynamic viscosity), ``nodes`` and ``inlet_scale`` (multiplies every
        prescribed inlet velocity) are optional differentiable parameters.
        """
        case, topo, dim = self.case, self.topo, self.dim
        nc = topo.n_cells
        # with node coordinates given, the SST wall distance follows the geometry too
        self._live_geometry = nodes is not None
        nodes = self.nodes if nodes is None else nodes
        geo = geometry(topo, nodes)
        m = Metrics(topo, geo)
        mu = torch.as_tensor(case["mu"], dtype=T) if mu is None else mu
        rho = case["rho"]
        bc_vel = self.bc_vel
        if inlet_scale is not None:
            bc_vel = torch.where((self.kind == 2)[:, None], bc_vel * inlet_scale, bc_vel)
        saved_vel = self.bc_vel
        self.bc_vel = bc_vel
        try:
            return self._residual(state, geo, m, mu, rho, nc, dim, return_fields)
        finally:
            self.bc_vel = saved_vel

    def _residual(self, state, geo, m, mu, rho, nc, dim, return_fields):
        case, topo = self.case, self.topo
        sst = case["sst"]
        n_flow = (dim + 1) * nc
        flow = state[:n_flow]
        u = flow[: dim * nc].reshape(dim, nc).T
        p = flow[dim * nc:]
        area, normal, vol = geo["area"], geo["normal"], geo["volume"]
        o = topo.owner
        rho_c = torch.full((nc,), rho, dtype=T)
        mu_c = mu * torch.ones(nc, dtype=T)

        # boundary values (leading order) and gradients, momentum.py:445-529, 822-857
        bvel = self._boundary_velocity(u)
        bp = self._boundary_pressure(p)
        gs = case.get("gradient")
        grad_u = torch.stack([gg_gradient(m, u[:, i], bvel[:, i], gs) for i in range(dim)], dim=1)
        grad_p = gg_gradient(m, p, bp, gs)

        visc = mu_c
        boundary_visc = None
        fields = {}
        log_k, log_w = (t == "log" for t in case.get("transforms", ("direct", "direct")))
        if sst is not None:
            # CoupledRANS.physical_fields (coupled.py:366-381): exp of a log-solved block
            k = state[n_flow:n_flow + nc]
            w = state[n_flow + nc:]
            k = torch.exp(k) if log_k else k
            w = torch.exp(w) if log_w else w
            nu = (mu / rho) * torch.ones(nc, dtype=T)
            dist, dgrad = self.wall_d, self.wall_dgrad
            if self._live_geometry:
                if self._nearest is None:
                    self._nearest = nearest_wall_face(case, geometry(topo, self.nodes))
                dist, dgrad = wall_distance_live(case, geo, m, self._nearest)
            wc = torch.as_tensor(sst["wall_cells"])
            wf = torch.as_tensor(sst["wall_faces"])
            # closure_fields, transport.py:548-579
            strain = strain_rate_magnitude(grad_u)
            wgt = wall_function_weight(nu[wc], dist[wc], k[wc])
            strain = strain.index_copy(0, wc, (1.0 - wgt) * strain[wc]
                                       + wgt * log_layer_shear_rate(dist[wc], k[wc]))
            kb0 = self._scalar_bvals(k, None, sst["k_kind"], sst["k_val"], geo)
            grad_k = gg_gradient(m, k, kb0, gs)
            wb0 = self._scalar_bvals(w, None, sst["omega_kind"], sst["omega_val"], geo)
            grad_w_rec = gg_gradient(m, w, wb0, gs)
            imposed = _omega_wall_gradient_live(nu[wc], dist[wc], k[wc], dgrad[wc], grad_k[wc])
            grad_w = grad_w_rec.index_copy(0, wc, imposed)
            f1 = sst_f1(k, w, nu, dist, grad_k, grad_w)
            nut = sst_nut(k, w, strain, nu, dist)
            # wall shear rate per wall cell, transport.py:508-546
            ow = o[wf]
            slip = u[ow] - bvel[wf]
            rate = safe_sqrt(_dot(slip, slip)) / dist[ow]
            zeros = torch.zeros(topo.n_faces, dtype=T)
            a_w = zeros.index_copy(0, wf, area[wf])
            weighted = zeros.index_copy(0, wf, rate) * a_w
            shear = topo.scatter(weighted, zeros)[wc] / topo.scatter(a_w, zeros)[wc]
            # momentum.with_eddy_viscosity, momentum.py:314-403
            nut_wall_face = zeros.index_copy(0, wf, nut_wall(nu[ow], dist[ow], k[ow]))
            visc = mu_c + rho_c * nut
            shears = (self.kind == 0) | (self.kind == 1)
            wall_mu = mu_c[o] + rho_c[o] * nut_wall_face
            boundary_visc = torch.where(shears, wall_mu, visc[o])

        # momentum_matrix_diagonal, momentum.py:596-693 + rhie_chow.py:81-271
        mom = rho_c[:, None] * u
        grad_mom = rho_c[:, None, None] * grad_u
        mom_n = _dot(interpolate_to_face(m, mom, grad_mom), normal)
        mdot_est = mom_n * area
        bvisc = visc[o] if boundary_visc is None else boundary_visc
        viscous_owner = bvisc * area / m.normal_distance
        conv_owner = torch.clamp(mdot_est, min=0.0)
        kind = self.kind
        bcoef = torch.where((kind == 0) | (kind == 1), viscous_owner,
                            torch.where(kind == 2, viscous_owner + conv_owner,
                                        torch.where(kind == 3, conv_owner, torch.zeros_like(area))))
        g_o, g_n = visc[o], visc[topo.safe_nb]
        denom = torch.where(topo.interior, m.dpn - g_o / g_n * m.dnn, m.dpn)
        viscous = g_o * area / denom
        own_c = viscous + torch.clamp(mdot_est, min=0.0)
        nb_c = viscous + torch.clamp(-mdot_est, min=0.0)
        own_c = torch.where(topo.interior, own_c, bcoef)
        a_p = topo.scatter(own_c, nb_c)
        d_coeff = (vol / a_p)[:, None].expand(nc, dim)

        # Rhie-Chow mass flux, rhie_chow.py:274-353 and flow/boundary.py:381-435
        rho_face = topo.blend(rho_c, rho_c, m.g)
        gp_face = topo.blend(grad_p, grad_p, m.g)
        dc_face = topo.blend(d_coeff, d_coeff, m.g)
        d_hat = _dot(normal * normal, dc_face)
        dp = p[topo.safe_nb] - p[o]
        damping = (dp - _dot(gp_face, m.d)) / m.normal_distance
        mdot_int = (mom_n - rho_face * d_hat * damping) * area
        mdot = torch.where(topo.interior, mdot_int, torch.zeros_like(mdot_int))
        inlet = rho_c[o] * _dot(self.bc_vel, normal) * area
        u_n = _dot(u[o], normal)
        compact = (self.bc_p - p[o]) / m.normal_distance
        interp = _dot(grad_p[o], normal)
        dh_o = _dot(normal * normal, d_coeff[o])
        outlet = rho_c[o] * (u_n - dh_o * (compact - interp)) * area
        mdot = torch.where(kind == 2, inlet, torch.where(kind == 3, outlet,
                                                          torch.where(kind >= 0, torch.zeros_like(mdot), mdot)))

        # momentum + continuity residual, momentum.py:498-511, 747-820
        p_face = torch.where(topo.interior, interpolate_to_face(m, p, grad_p), bp)
        cols = []
        for i in range(dim):
            diff = diffusion_flux(m, u[:, i], grad_u[:, i], visc, bvel[:, i], boundary_visc)
            press = p_face * normal[:, i] * area
            adv = advection_flux(m, u[:, i], grad_u[:, i], mdot, bvel[:, i],
                                 case.get("advection"))
            flux = ((torch.zeros_like(area) + diff) + press) + adv
            cols.append(topo.scatter_conservative(flux) - 0.0 * vol)
        r_cont = topo.scatter_conservative(mdot)
        if case["pin"] is not None:
            pin = case["pin"]
            r_cont = r_cont.index_copy(0, torch.tensor([pin]),
                                       (p[pin] - case["pin_value"]).reshape(1))
        out = [c for c in cols] + [r_cont]
        if return_fields:
            fields.update(grad_u=grad_u, grad_p=grad_p, mdot=mdot, a_p=a_p, bvel=bvel, bp=bp)
        if sst is None:
            r = torch.cat(out)
            return (r, fields) if return_fields else r

        # k equation, transport.py:581-653
        vflux = mdot / rho
        gam_k = nu + blend(f1, SIGMA_K1, SIGMA_K2) * nut
        kb = self._scalar_bvals(k, grad_k, sst["k_kind"], sst["k_val"], geo)
        face_gamma = gam_k[o]
        wfw = wall_function_weight(nu[ow], dist[ow], k[ow])
        face_gamma = face_gamma.index_copy(0, wf, (1.0 - wfw) * face_gamma[wf])
        sadv = case.get("scalar_advection", case.get("advection"))
        kflux = (torch.zeros_like(area) + advection_flux(m, k, grad_k, vflux, kb, sadv)) + \
            diffusion_flux(m, k, grad_k, gam_k, kb, face_gamma)
        r_k = topo.scatter_conservative(kflux)
        prod = nut * strain ** 2
        limit = PRODUCTION_LIMIT_RATIO * BETA_STAR * torch.clamp(k, min=0.0) * w
        limited = torch.minimum(prod, limit)
        kw = k[wc]
        lw = wall_function_weight(nu[wc], dist[wc], kw)
        tau = (nu[wc] + nut_wall(nu[wc], dist[wc], kw)) * shear
        pw = tau * log_layer_shear_rate(dist[wc], kw)
        limited = limited.index_copy(0, wc, (1.0 - lw) * limited[wc] + lw * pw)
        r_k = r_k - limited * vol
        w_eff = w.index_copy(0, wc, omega_wall(nu[wc], dist[wc], kw))
        r_k = r_k - (-BETA_STAR * k * w_eff * vol)

        # omega equation, transport.py:655-718
        gam_w = nu + blend(f1, SIGMA_W1, SIGMA_W2) * nut
        wb = self._scalar_bvals(w, grad_w_rec, sst["omega_kind"], sst["omega_val"], geo)
        wflux = (torch.zeros_like(area) + advection_flux(m, w, grad_w_rec, vflux, wb, sadv)) + \
            diffusion_flux(m, w, grad_w_rec, gam_w, wb)
        r_w = topo.scatter_conservative(wflux)
        alpha = blend(f1, ALPHA_1, ALPHA_2)
        cap = PRODUCTION_LIMIT_RATIO * BETA_STAR * torch.clamp(k, min=0.0) * w / \
            torch.clamp(nut, min=EDDY_VISCOSITY_FLOOR)
        r_w = r_w - alpha * torch.minimum(strain ** 2, cap) * vol
        beta = blend(f1, BETA_1, BETA_2)
        r_w = r_w - (-beta * w ** 2 * vol)
        cross = 2.0 * (1.0 - f1) * SIGMA_W2 * _dot(grad_k, grad_w) / w
        r_w = r_w - cross * vol
        # FixedValueCells with the transform's fixation row (fixed_value.py:80-158): the plain
        # difference, or the log ratio for a log-solved omega
        target = omega_wall(nu[wc], dist[wc], k[wc])
        fix = torch.log(w[wc] / target) if log_w else w[wc] - target
        r_w = r_w.index_copy(0, wc, fix)
        r = torch.cat(out + [r_k, r_w])
        if return_fields:
            fields.update(strain=strain, f1=f1, nut=nut, grad_k=grad_k, grad_w=grad_w, shear=shear)
            return r, fields
        return r

    def jvp(self, state, direction):
        """``J v`` by reverse-over-reverse AD (exact; torch's forward mode is not used because one
        of its rules disagreed with reverse mode and with Richardson finite differences)."""
        s = _t(state).requires_grad_(True)
        r = self.residual(s)
        u = torch.zeros_like(r, requires_grad=True)
        (g,) = torch.autograd.grad(r, s, u, create_graph=True)
        (jv,) = torch.autograd.grad(g, u, _t(direction))
        return jv.detach()

    def vjp(self, state, cotangent):
        s = _t(state).requires_grad_(True)
        r = self.residual(s)
        (g,) = torch.autograd.grad(r, s, _t(cotangent))
        return g
