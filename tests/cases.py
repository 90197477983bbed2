"""Golden-fixture loaders and the case descriptions shared by the CPU and GPU tests."""
from __future__ import annotations

import os
import types

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_cache: dict = {}


def golden(name: str):
    if name not in _cache:
        _cache[name] = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    return _cache[name]


def mesh_from(d: dict, prefix: str):
    """A mesh namespace (nodes, CSR face nodes, owner/neighbour, patches) from fixture arrays."""
    patches = {k[len(prefix) + 6:]: d[k] for k in d if k.startswith(prefix + "patch_")}
    return types.SimpleNamespace(
        nodes=d[prefix + "nodes"], fn_offsets=d[prefix + "fn_offsets"],
        fn_indices=d[prefix + "fn_indices"], owner=d[prefix + "owner"],
        neighbour=d[prefix + "neighbour"], n_cells=len(d[prefix + "volume"]), patches=patches)


CAVITY_BC = {"top": ("moving", (1.0, 0.0)), "bottom": ("wall",), "left": ("wall",),
             "right": ("wall",)}
DUCT3_BC = {"left": ("inlet", (1.0, 0.0, 0.0)), "right": ("outlet", 0.0), "bottom": ("wall",),
            "top": ("wall",), "back": ("wall",), "front": ("wall",)}


def sst_spec(dim, nu, k_in, w_in, walls, k_wall=("dirichlet", 0.0)):
    fb = {"left": ("inlet", (1.0,) + (0.0,) * (dim - 1)), "right": ("outlet", 0.0)}
    fb.update({w: ("wall",) for w in walls})
    kb = {"left": ("dirichlet", k_in), "right": ("zerograd",)}
    kb.update({w: tuple(k_wall) for w in walls})
    wb = {"left": ("dirichlet", w_in), "right": ("zerograd",)}
    wb.update({w: ("zerograd",) for w in walls})
    return fb, {"nu": nu, "walls": list(walls), "k": kb, "omega": wb}


# (fixture file, prefix, description) of every residual case pinned by the reference.
# Cases with a ``gradient`` entry use corrected Green-Gauss by swept sweeps (fixture "corrected").
LAMINAR = {
    "cav8": dict(prefix="cav8_", mu=0.01, bc=CAVITY_BC, pin=0),
    "cavj": dict(prefix="cavj_", mu=0.01, bc=CAVITY_BC, pin=0),
    "lam3": dict(prefix="lam3_", mu=0.02, bc=DUCT3_BC, pin=None),
    "ccavj": dict(prefix="ccavj_", mu=0.01, bc=CAVITY_BC, pin=0, file="corrected",
                  gradient={"sweeps": 4, "relaxation": 1.0}),
    "lcavj": dict(prefix="lcavj_", mu=0.01, bc=CAVITY_BC, pin=0, file="limited",
                  advection={"k": 5.0}),
    "ucavj": dict(prefix="ucavj_", mu=0.01, bc=CAVITY_BC, pin=0, file="limited",
                  advection={"k": None}),
}
SST = {
    "sst2": dict(prefix="sst2_", dim=2, nu=2e-5, walls=["bottom", "top"]),
    "sst3": dict(prefix="sst3_", dim=3, nu=1e-3, walls=["bottom", "top", "back", "front"]),
    "csst2": dict(prefix="csst2_", dim=2, nu=2e-5, walls=["bottom", "top"], file="corrected",
                  gradient={"sweeps": 4, "relaxation": 1.0}),
    "csst3": dict(prefix="csst3_", dim=3, nu=1e-3, walls=["bottom", "top", "back", "front"],
                  file="corrected", gradient={"sweeps": 3, "relaxation": 0.8}),
    "lsst2": dict(prefix="lsst2_", dim=2, nu=2e-5, walls=["bottom", "top"], file="limited",
                  advection={"k": 5.0}),
    # LogScalars: log omega (2D), log k and log omega (3D); states hold the solved variables
    "wsst2": dict(prefix="wsst2_", dim=2, nu=2e-5, walls=["bottom", "top"], file="logscalars",
                  transforms=("direct", "log")),
    "bsst3": dict(prefix="bsst3_", dim=3, nu=1e-3, walls=["bottom", "top", "back", "front"],
                  file="logscalars", transforms=("log", "log")),
    # the backward-step validation configuration: limited momentum, upwind k / omega, corrected
    # gradients, zero-gradient k walls, log omega; and the reverse advection split
    "psst2": dict(prefix="psst2_", dim=2, nu=2e-5, walls=["bottom", "top"], file="mixed",
                  advection={"k": 5.0}, scalar_advection="upwind",
                  gradient={"sweeps": 4, "relaxation": 1.0}, k_wall=("zerograd",),
                  transforms=("direct", "log")),
    "msst2": dict(prefix="msst2_", dim=2, nu=2e-5, walls=["bottom", "top"], file="mixed",
                  scalar_advection={"k": 5.0}),
}


def oracle_case(name: str):
    """(oracle case dict, fixture dict, prefix) for a named golden residual case."""
    from oracle import fv_oracle as fo

    if name in LAMINAR:
        spec = LAMINAR[name]
        d = golden(spec.get("file", "laminar"))
        mesh = mesh_from(d, spec["prefix"])
        case = fo.make_case(mesh, mu=spec["mu"], rho=1.0, flow_bc=spec["bc"],
                            pressure_pin=spec["pin"], gradient=spec.get("gradient"),
                            advection=spec.get("advection"))
        return case, d, spec["prefix"]
    spec = SST[name]
    d = golden(spec.get("file", "sst"))
    mesh = mesh_from(d, spec["prefix"])
    k_in, w_in = d[spec["prefix"] + "inlet"]
    fb, sst = sst_spec(spec["dim"], spec["nu"], float(k_in), float(w_in), spec["walls"],
                       spec.get("k_wall", ("dirichlet", 0.0)))
    case = fo.make_case(mesh, mu=spec["nu"], rho=1.0, flow_bc=fb, sst=sst,
                        gradient=spec.get("gradient"), advection=spec.get("advection"),
                        scalar_advection=spec.get("scalar_advection"),
                        transforms=spec.get("transforms", ("direct", "direct")))
    return case, d, spec["prefix"]


def mesh_data(d: dict, prefix: str):
    """The fixture mesh as the package's :class:`MeshData`."""
    from aquaflux_gb300.mesh import MeshData

    ns = mesh_from(d, prefix)
    return MeshData(nodes=np.ascontiguousarray(ns.nodes, dtype=np.float64),
                    fn_offsets=ns.fn_offsets.astype(np.int32), fn_indices=ns.fn_indices.astype(np.int32),
                    owner=ns.owner.astype(np.int32), neighbour=ns.neighbour.astype(np.int32),
                    n_cells=int(ns.n_cells), patches={k: v.astype(np.int32) for k, v in ns.patches.items()})


def device_case(name: str):
    """(FlowCase on the GPU, oracle case dict, fixture dict, prefix) for a golden case."""
    from aquaflux_gb300 import fv

    case, d, p = oracle_case(name)
    m = mesh_data(d, p)
    dm = fv.DeviceMesh(m)
    if name in LAMINAR:
        spec = LAMINAR[name]
        fc = fv.FlowCase(dm, mu=spec["mu"], rho=1.0, flow_bc=spec["bc"], pressure_pin=spec["pin"],
                         gradient=spec.get("gradient"), advection=spec.get("advection"))
    else:
        spec = SST[name]
        k_in, w_in = d[p + "inlet"]
        fb, sst = sst_spec(spec["dim"], spec["nu"], float(k_in), float(w_in), spec["walls"],
                           spec.get("k_wall", ("dirichlet", 0.0)))
        k_tr, w_tr = spec.get("transforms", ("direct", "direct"))
        fc = fv.FlowCase(dm, mu=spec["nu"], rho=1.0, flow_bc=fb, sst=sst,
                         gradient=spec.get("gradient"), advection=spec.get("advection"),
                         k_transform=k_tr, omega_transform=w_tr,
                         scalar_advection=spec.get("scalar_advection"))
    return fc, case, d, p


def workload_oracle_case(wl):
    """The oracle's case dict for a :class:`aquaflux_gb300.workloads.Workload`."""
    from oracle import fv_oracle as fo

    sst = None
    if wl.sst is not None:
        sst = {"nu": wl.mu / wl.rho, "walls": wl.sst["walls"], "k": wl.sst["k"],
               "omega": wl.sst["omega"]}
    return fo.make_case(wl.mesh, mu=wl.mu, rho=wl.rho, flow_bc=wl.flow_bc,
                        pressure_pin=wl.pressure_pin, sst=sst, gradient=wl.gradient,
                        advection=wl.advection, scalar_advection=wl.scalar_advection,
                        transforms=(wl.k_transform, wl.omega_transform))
