"""The oracle's Newton (exact sparse Jacobian from reverse-mode products, sparse LU): its Jacobian
reproduces the oracle's J v, and it converges the small cavity from rest to the reference's
tolerance -- the checker of the GPU Newton solve, pinned here on the CPU."""
import numpy as np
import torch

from aquaflux_gb300 import mesh as fm
from oracle import fv_oracle as fo
from oracle.newton_oracle import OracleJacobian, greedy_colouring, newton

CAVITY_BC = {"top": ("moving", (1.0, 0.0)), "bottom": ("wall",), "left": ("wall",),
             "right": ("wall",)}


def _case(n):
    m = fm.structured_grid_2d(n, n)
    return m, fo.Oracle(fo.make_case(m, mu=0.01, rho=1.0, flow_bc=CAVITY_BC, pressure_pin=0))


def test_colouring_separates_rows_sharing_a_column():
    m, orc = _case(10)
    jac = OracleJacobian(orc, m.owner, m.neighbour, 100, 3)
    conflict = (jac.pat.T @ jac.pat).tocoo()
    off = conflict.row != conflict.col
    assert np.all(jac.colour[conflict.row[off]] != jac.colour[conflict.col[off]])
    assert np.array_equal(greedy_colouring(jac.pat), jac.colour)


def test_sparse_jacobian_reproduces_the_oracle_jvp():
    m, orc = _case(10)
    jac = OracleJacobian(orc, m.owner, m.neighbour, 100, 3)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(300) * 0.2
    v = rng.standard_normal(300)
    jv = orc.jvp(x, v).numpy()
    assert np.abs(jac.matrix(x) @ v - jv).max() <= 1e-13 * np.abs(jv).max()


def test_oracle_newton_converges_the_cavity_from_rest():
    m, orc = _case(10)
    jac = OracleJacobian(orc, m.owner, m.neighbour, 100, 3)
    res = newton(orc, jac, np.zeros(300))
    assert res["converged"]
    assert res["residual_norms"][-1] <= 1e-12 + 1e-10 * res["residual_norms"][0]
    r = orc.residual(torch.as_tensor(res["state"])).numpy()
    assert np.linalg.norm(r) == res["residual_norms"][-1]
