"""The CPU oracle against golden vectors produced by the reference package itself.

These pin the oracle before it is trusted as the checker of the CUDA path: geometry, laminar and
SST residuals must agree with the reference to rounding, and the oracle's autograd JVP must agree
with central finite differences of the reference residual.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import fv_oracle as fo
from tests.cases import LAMINAR, SST, golden, mesh_from, oracle_case


@pytest.mark.parametrize("prefix", ["m2d_", "m3d_", "mgr_", "cav8_", "cavj_", "lam3_"])
def test_geometry_matches_reference(prefix):
    d = golden("meshes") if prefix.startswith("m") else golden("laminar")
    mesh = mesh_from(d, prefix)
    topo = fo.Topology(mesh.owner, mesh.neighbour, mesh.n_cells, mesh.fn_offsets, mesh.fn_indices)
    geo = fo.geometry(topo, torch.as_tensor(mesh.nodes))
    for key in ("area", "normal", "face_centroid", "volume", "cell_centroid"):
        ref = d[prefix + key]
        np.testing.assert_allclose(geo[key].numpy(), ref, rtol=0, atol=1e-14 * max(1.0, np.abs(ref).max()))


@pytest.mark.parametrize("name", list(LAMINAR) + list(SST))
def test_residual_matches_reference(name):
    case, d, p = oracle_case(name)
    orc = fo.Oracle(case)
    for state, ref in zip(d[p + "states"], d[p + "residuals"]):
        r = orc.residual(torch.as_tensor(state)).numpy()
        assert np.abs(r - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("name", ["cav8", "cavj", "lam3", "sst2", "sst3", "ccavj", "csst2", "lcavj",
                                  "ucavj", "lsst2"])
def test_jvp_matches_reference_finite_differences(name):
    case, d, p = oracle_case(name)
    orc = fo.Oracle(case)
    state = d[p + "states"][1 if name == "cav8" else 0]
    jv = orc.jvp(state, d[p + "jvp_dir"]).numpy()
    fd = d[p + "jvp_fd"]
    assert np.abs(jv - fd).max() <= 1e-7 * np.abs(fd).max()


def test_sst_wall_distance_matches_reference():
    for name in SST:
        case, d, p = oracle_case(name)
        if p + "wall_distance" not in d:
            continue
        orc = fo.Oracle(case)
        np.testing.assert_allclose(orc.wall_d.numpy(), d[p + "wall_distance"], rtol=1e-14)
        np.testing.assert_allclose(orc.wall_dgrad.numpy(), d[p + "wall_distance_gradient"],
                                   rtol=0, atol=1e-13)


@pytest.mark.parametrize("name", ["cav8_s1_", "cavj_s0_", "lam3_s0_"])
def test_intermediate_fields_match_reference(name):
    case_name = {"cav8_s1_": "cav8", "cavj_s0_": "cavj", "lam3_s0_": "lam3"}[name]
    case, d, p = oracle_case(case_name)
    orc = fo.Oracle(case)
    state = d[p + "states"][1 if case_name == "cav8" else 0]
    _, f = orc.residual(torch.as_tensor(state), return_fields=True)
    for key in ("grad_u", "grad_p", "mdot", "a_p", "bvel", "bp"):
        ref = d[name + key]
        np.testing.assert_allclose(f[key].numpy(), ref, rtol=0, atol=1e-13 * max(1.0, np.abs(ref).max()))


def test_vjp_is_the_transpose_of_jvp():
    case, d, p = oracle_case("sst2")
    orc = fo.Oracle(case)
    rng = np.random.default_rng(0)
    state = d[p + "states"][0]
    v = rng.standard_normal(state.size)
    w = rng.standard_normal(state.size)
    lhs = float(np.dot(w, orc.jvp(state, v).numpy()))
    rhs = float(np.dot(orc.vjp(state, w).numpy(), v))
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)


@pytest.mark.parametrize("sweeps,relax", [(4, 1.0), (24, 1.0), (6, 0.8)])
def test_corrected_gradient_matches_reference(sweeps, relax):
    """CorrectedGreenGauss + SweptGradientSolve on a jittered mesh, for a linear field (exact at
    convergence: 24 sweeps) and a random field with random boundary values."""
    d = golden("corrected")
    mesh = mesh_from(d, "g2_")
    topo = fo.Topology(mesh.owner, mesh.neighbour, mesh.n_cells, mesh.fn_offsets, mesh.fn_indices)
    m = fo.Metrics(topo, fo.geometry(topo, torch.as_tensor(mesh.nodes)))
    for f, b, ref in zip(d["g2_fields"], d["g2_bvals"], d[f"g2_grad_s{sweeps}"]):
        g = fo.gg_gradient(m, torch.as_tensor(f), torch.as_tensor(b),
                           {"sweeps": sweeps, "relaxation": relax}).numpy()
        assert np.abs(g - ref).max() <= 1e-13 * np.abs(ref).max()
    if sweeps == 24:
        np.testing.assert_allclose(d["g2_grad_s24"][0], np.tile([1.3, -2.1], (mesh.n_cells, 1)),
                                   rtol=0, atol=1e-13)


def test_corrected_intermediate_fields_match_reference():
    case, d, p = oracle_case("ccavj")
    orc = fo.Oracle(case)
    _, f = orc.residual(torch.as_tensor(d[p + "states"][0]), return_fields=True)
    for key in ("grad_u", "grad_p", "mdot", "a_p", "bvel", "bp"):
        ref = d["ccavj_s0_" + key]
        np.testing.assert_allclose(f[key].numpy(), ref, rtol=0,
                                   atol=1e-13 * max(1.0, np.abs(ref).max()))
