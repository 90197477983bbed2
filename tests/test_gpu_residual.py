"""CUDA residual / JVP against the CPU oracle and the reference's golden vectors."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import fv_oracle as fo
from tests.cases import LAMINAR, SST, device_case, golden, mesh_data, oracle_case

pytestmark = pytest.mark.gpu
ALL = list(LAMINAR) + list(SST)


def _rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("prefix", ["m2d_", "m3d_", "mgr_", "cav8_", "cavj_", "lam3_"])
def test_geometry_matches_reference(prefix):
    from aquaflux_gb300 import fv

    d = golden("meshes") if prefix.startswith("m") else golden("laminar")
    dm = fv.DeviceMesh(mesh_data(d, prefix))
    geo = dm.geometry()
    for key in ("area", "normal", "face_centroid", "volume", "cell_centroid"):
        ref = d[prefix + key]
        got = geo[key].cpu().numpy()
        assert np.abs(got - ref).max() <= 1e-14 * max(1.0, np.abs(ref).max()), key


@pytest.mark.parametrize("name", ALL)
def test_residual_matches_reference_golden(name):
    fc, case, d, p = device_case(name)
    for state, ref in zip(d[p + "states"], d[p + "residuals"]):
        assert _rel(fc.residual(state), ref) <= 1e-12


@pytest.mark.parametrize("name", ALL)
def test_residual_matches_oracle_at_fresh_states(name):
    fc, case, d, p = device_case(name)
    orc = fo.Oracle(case)
    rng = np.random.default_rng(5)
    base = d[p + "states"][0]
    for _ in range(2):
        s = base * (1.0 + 0.1 * rng.standard_normal(base.size))
        ref = orc.residual(torch.as_tensor(s)).numpy()
        assert _rel(fc.residual(s), ref) <= 1e-12


@pytest.mark.parametrize("name", ALL)
def test_jvp_matches_oracle(name):
    fc, case, d, p = device_case(name)
    orc = fo.Oracle(case)
    rng = np.random.default_rng(7)
    s = d[p + "states"][0]
    v = rng.standard_normal(s.size) * (np.abs(s) + 1e-3)
    r, jv = fc.jvp(s, v, return_residual=True)
    assert _rel(jv, orc.jvp(s, v).numpy()) <= 1e-11
    assert _rel(r, orc.residual(torch.as_tensor(s)).numpy()) <= 1e-12


@pytest.mark.parametrize("name", ["cav8", "lam3", "sst2", "sst3", "ccavj", "csst2", "lcavj", "ucavj",
                                  "lsst2", "wsst2", "bsst3", "psst2", "msst2"])
def test_jvp_matches_reference_finite_differences(name):
    fc, case, d, p = device_case(name)
    s = d[p + "states"][1 if name == "cav8" else 0]
    jv = fc.jvp(s, d[p + "jvp_dir"])
    assert _rel(jv, d[p + "jvp_fd"]) <= 1e-7


@pytest.mark.parametrize("name", ["cavj", "lam3", "sst2", "ccavj", "csst3", "wsst2", "bsst3"])
def test_parameter_jvp_matches_oracle(name):
    fc, case, d, p = device_case(name)
    orc = fo.Oracle(case)
    s = torch.as_tensor(d[p + "states"][0])
    mu = torch.tensor(case["mu"], dtype=torch.float64, requires_grad=True)
    scale = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    dmu_gpu, dsc_gpu = fc.param_jvp(s.numpy())
    w = torch.randn(s.numel(), dtype=torch.float64)
    r = orc.residual(s, mu=mu, inlet_scale=scale)
    gmu, gsc = torch.autograd.grad((r * w).sum(), (mu, scale), allow_unused=True)
    assert abs(float((dmu_gpu.cpu() * w).sum()) - float(gmu)) <= 1e-10 * max(1.0, abs(float(gmu)))
    gsc = 0.0 if gsc is None else float(gsc)
    assert abs(float((dsc_gpu.cpu() * w).sum()) - gsc) <= 1e-10 * max(1.0, abs(gsc))


def test_zero_state_jvp_uses_the_tie_rule():
    """At the zero state every mass flux is exactly 0; max(mdot, 0) takes half the tangent (JAX)."""
    fc, case, d, p = device_case("cav8")
    z = np.zeros(fc.n_unknowns)
    rng = np.random.default_rng(3)
    v = rng.standard_normal(z.size)
    jv = fc.jvp(z, v).cpu().numpy()
    h = 1e-7
    r_plus = fc.residual(h * v).cpu().numpy()
    r_minus = fc.residual(-h * v).cpu().numpy()
    central = (r_plus - r_minus) / (2 * h)
    assert np.abs(jv - central).max() <= 1e-6 * np.abs(central).max()


@pytest.mark.parametrize("name", ["cav8", "sst3", "csst3"])
def test_run_to_run_bitwise_identical(name):
    fc, case, d, p = device_case(name)
    s = d[p + "states"][0]
    a = fc.residual(s).cpu().numpy()
    b = fc.residual(s).cpu().numpy()
    assert np.array_equal(a, b)
    v = np.ones(s.size)
    assert np.array_equal(fc.jvp(s, v).cpu().numpy(), fc.jvp(s, v).cpu().numpy())


@pytest.mark.parametrize("name", [n for n in SST if n != "lsst2"])
def test_wall_distance_matches_reference(name):
    fc, case, d, p = device_case(name)
    wd, wdg = fc.wall_distance()
    np.testing.assert_allclose(wd.cpu().numpy(), d[p + "wall_distance"], rtol=1e-14)
    np.testing.assert_allclose(wdg.cpu().numpy(), d[p + "wall_distance_gradient"], rtol=0, atol=1e-13)


def test_config1_cavity_64_matches_reference():
    from aquaflux_gb300 import fv, mesh as fm

    d = golden("laminar")
    m = fm.structured_grid_2d(64, 64)
    fc = fv.FlowCase(fv.DeviceMesh(m), mu=0.01, rho=1.0, pressure_pin=0,
                     flow_bc={"top": ("moving", (1.0, 0.0)), "bottom": ("wall",),
                              "left": ("wall",), "right": ("wall",)})
    for s, ref in zip(d["cav64_states"], d["cav64_residuals"]):
        assert _rel(fc.residual(s), ref) <= 1e-12


def test_bad_state_shape_rejected():
    fc, case, d, p = device_case("cav8")
    with pytest.raises(ValueError):
        fc.residual(np.zeros(fc.n_unknowns + 1))


@pytest.mark.parametrize("name", ALL)
def test_vjp_matches_oracle(name):
    fc, case, d, p = device_case(name)
    orc = fo.Oracle(case)
    rng = np.random.default_rng(11)
    for s in d[p + "states"][:2]:
        w = rng.standard_normal(s.size)
        r, g = fc.vjp(s, w, return_residual=True)
        ref = orc.vjp(s, w).numpy()
        assert _rel(g, ref) <= 1e-11, name
        assert _rel(r, orc.residual(torch.as_tensor(s)).numpy()) <= 1e-12


@pytest.mark.parametrize("name", ALL)
def test_vjp_is_the_transpose_of_jvp_on_gpu(name):
    fc, case, d, p = device_case(name)
    rng = np.random.default_rng(13)
    s = d[p + "states"][0]
    v = rng.standard_normal(s.size)
    w = rng.standard_normal(s.size)
    jv = fc.jvp(s, v).cpu().numpy()
    g = fc.vjp(s, w).cpu().numpy()
    lhs, rhs = float(np.dot(w, jv)), float(np.dot(g, v))
    scale = float(np.abs(w * jv).sum())
    assert abs(lhs - rhs) <= 1e-12 * scale


@pytest.mark.parametrize("name", ["cavj", "lam3", "sst2", "sst3", "ccavj", "csst2", "csst3", "wsst2",
                                  "bsst3"])
def test_param_vjp_matches_oracle(name):
    fc, case, d, p = device_case(name)
    orc = fo.Oracle(case)
    s = torch.as_tensor(d[p + "states"][0])
    w = torch.randn(s.numel(), dtype=torch.float64)
    mu = torch.tensor(case["mu"], dtype=torch.float64, requires_grad=True)
    scale = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    r = orc.residual(s, mu=mu, inlet_scale=scale)
    gmu, gsc = torch.autograd.grad((r * w).sum(), (mu, scale), allow_unused=True)
    got = fc.param_vjp(s.numpy(), w.numpy()).cpu().numpy()
    assert abs(got[0] - float(gmu)) <= 1e-10 * max(1.0, abs(float(gmu)))
    gsc = 0.0 if gsc is None else float(gsc)
    assert abs(got[1] - gsc) <= 1e-10 * max(1.0, abs(gsc))


def test_vjp_at_negative_k_and_zero_state():
    """Clamped k (max(k, 0)) and the zero state's mass-flux ties take the forward subgradients."""
    fc, case, d, p = device_case("sst2")
    orc = fo.Oracle(case)
    s = d[p + "states"][2]  # contains negative k cells
    w = np.random.default_rng(17).standard_normal(s.size)
    assert _rel(fc.vjp(s, w), orc.vjp(s, w).numpy()) <= 1e-11
    fc0, case0, d0, p0 = device_case("cav8")
    z = np.zeros(fc0.n_unknowns)
    v = np.random.default_rng(19).standard_normal(z.size)
    w = np.random.default_rng(23).standard_normal(z.size)
    lhs = float(np.dot(w, fc0.jvp(z, v).cpu().numpy()))
    rhs = float(np.dot(fc0.vjp(z, w).cpu().numpy(), v))
    assert abs(lhs - rhs) <= 1e-12 * max(1.0, abs(lhs))


@pytest.mark.parametrize("sweeps,relax", [(1, 1.0), (1, 0.7), (2, 1.0), (5, 0.8), (24, 1.0)])
def test_corrected_gradient_sweep_counts(sweeps, relax):
    """Odd and even sweep counts, the peel alone and under-relaxation: residual, JVP and VJP against
    the oracle on the jittered cavity (the ping-pong of the sweep iterates ends in the right
    buffer for every count)."""
    from aquaflux_gb300 import fv

    case, d, p = oracle_case("cavj")
    case = dict(case, gradient={"sweeps": sweeps, "relaxation": relax})
    fc = fv.FlowCase(fv.DeviceMesh(mesh_data(d, p)), mu=0.01, rho=1.0,
                     flow_bc=LAMINAR["cavj"]["bc"], pressure_pin=0,
                     gradient={"sweeps": sweeps, "relaxation": relax})
    orc = fo.Oracle(case)
    s = d[p + "states"][1]
    assert _rel(fc.residual(s), orc.residual(torch.as_tensor(s)).numpy()) <= 1e-12
    rng = np.random.default_rng(sweeps)
    v = rng.standard_normal(s.size)
    assert _rel(fc.jvp(s, v), orc.jvp(s, v).numpy()) <= 1e-11
    w = rng.standard_normal(s.size)
    assert _rel(fc.vjp(s, w), orc.vjp(s, w).numpy()) <= 1e-11


def test_corrected_scheme_rejects_bad_relaxation():
    from aquaflux_gb300 import fv
    from aquaflux_gb300._lib import FvError

    case, d, p = oracle_case("cavj")
    dm = fv.DeviceMesh(mesh_data(d, p))
    for bad in ({"sweeps": 3, "relaxation": 0.0}, {"sweeps": 3, "relaxation": 1.5},
                {"sweeps": -1, "relaxation": 1.0}):
        with pytest.raises(FvError):
            fv.FlowCase(dm, mu=0.01, rho=1.0, flow_bc=LAMINAR["cavj"]["bc"], gradient=bad)
