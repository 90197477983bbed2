"""The mesh-coordinate adjoint d/dnodes (w . R) against the oracle's autograd through the geometry
(laminar 2D / 3D, k-omega SST 2D / 3D with the wall distance following the nodes, the corrected
Green-Gauss scheme's swept solve for the fields and the wall-distance gradient, the limited and
unlimited linear-upwind reconstruction with the Venkatakrishnan limiter, the backward-step
validation configuration) and against central differences of the GPU residual under moved nodes
(laminar: compact, corrected, limited)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import fv_oracle as fo
from tests.cases import device_case

pytestmark = pytest.mark.gpu


def _oracle_node_grad(case, d, p, s, w):
    orc = fo.Oracle(case)
    nodes = torch.tensor(d[p + "nodes"], dtype=torch.float64, requires_grad=True)
    r = orc.residual(torch.as_tensor(s), nodes=nodes)
    (g,) = torch.autograd.grad((r * torch.as_tensor(w)).sum(), nodes)
    return g.numpy()


@pytest.mark.parametrize("name", ["cav8", "cavj", "lam3", "sst2", "sst3", "wsst2", "bsst3",
                                  "ccavj", "csst2", "csst3", "lcavj", "ucavj", "lsst2", "psst2",
                                  "msst2"])
def test_node_vjp_matches_oracle_autograd(name):
    fc, case, d, p = device_case(name)
    s = d[p + "states"][0 if name != "cav8" else 1]
    w = np.random.default_rng(2).standard_normal(s.size)
    got = fc.node_vjp(s, w).cpu().numpy()
    ref = _oracle_node_grad(case, d, p, s, w)
    scale = np.abs(ref).max()
    assert np.abs(got - ref).max() <= 1e-10 * scale, (name, np.abs(got - ref).max() / scale)


@pytest.mark.parametrize("name", ["cavj", "ccavj", "lcavj"])
def test_node_vjp_matches_central_differences(name):
    """Jittered cavity (compact; corrected, 4 sweeps; limited): (w . R(x + h v) - w . R(x - h v)) / 2h
    against dnodes . v, the residual re-evaluated on the GPU after moving the nodes (geometry
    recomputed there)."""
    from aquaflux_gb300._lib import check, lib, ptr

    fc, case, d, p = device_case(name)
    s = d[p + "states"][0]
    rng = np.random.default_rng(4)
    w = rng.standard_normal(s.size)
    nodes = d[p + "nodes"]
    v = rng.standard_normal(nodes.shape) * 1e-2
    g = fc.node_vjp(s, w).cpu().numpy()
    h = 1e-6

    def wr(x):
        xd = torch.tensor(x, device="cuda")
        check(lib().fv_mesh_set_nodes(fc.dmesh.handle, ptr(xd), torch.cuda.current_stream().cuda_stream))
        return float(np.dot(w, fc.residual(s).cpu().numpy()))

    fd = (wr(nodes + h * v) - wr(nodes - h * v)) / (2 * h)
    wr(nodes)
    exact = float((g * v).sum())
    assert abs(fd - exact) <= 1e-6 * max(abs(exact), 1.0)


def test_node_vjp_refuses_a_caller_set_wall_distance():
    from aquaflux_gb300._lib import FvError

    fc, case, d, p = device_case("sst2")
    dist, _ = fc.wall_distance()
    fc.set_wall_distance(dist)
    with pytest.raises(FvError):
        fc.node_vjp(d[p + "states"][0], np.ones(fc.n_unknowns))
