"""The device FGMRES (``fv_krylov_*`` kernels: CGS2 projections, Hessenberg column, Givens
reduction and residual estimate on the GPU, the host reading the estimates one iteration late)
against the plain-torch checker in ``tests/krylov_reference.py``: same iteration counts and
convergence, solutions within rounding, bitwise identical run to run; restarts, the iteration cap,
a longer basis than one launch handles, exact breakdowns."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from tests.krylov_reference import fgmres_reference

pytestmark = pytest.mark.gpu


def _system(n, seed, spread=0.1, diag=4.0):
    rng = np.random.default_rng(seed)
    a = np.eye(n) * diag + rng.standard_normal((n, n)) / np.sqrt(n)
    a[np.tril_indices(n, -3)] *= spread
    return (torch.tensor(a, device="cuda"), torch.tensor(rng.standard_normal(n), device="cuda"))


@pytest.mark.parametrize("n,restart,maxiter,rtol", [(60, 30, 300, 1e-10), (60, 5, 300, 1e-10),
                                                    (300, 30, 300, 1e-3), (60, 4, 9, 1e-12),
                                                    (2000, 40, 200, 1e-11)])
def test_device_fgmres_matches_the_reference(n, restart, maxiter, rtol):
    from aquaflux_gb300.solve import fgmres

    # the 2000-unknown system converges slowly enough to pass 32 basis vectors (chunked launches)
    a, b = _system(n, 0, spread=1.0, diag=2.0) if n == 2000 else _system(n, 0)
    d = torch.diagonal(a).clone()

    def mv(v):
        return a @ v

    def jacobi(v):
        return v / d

    got = fgmres(mv, b, jacobi, rtol=rtol, restart=restart, maxiter=maxiter)
    x, its, res, conv = fgmres_reference(mv, b, jacobi, rtol=rtol, restart=restart,
                                         maxiter=maxiter)
    assert (got.iterations, got.converged) == (its, conv)
    assert torch.allclose(got.x, x, rtol=1e-9, atol=1e-12 * float(x.abs().max()))
    assert abs(got.residual_norm - res) <= 1e-6 * res + 1e-14
    # bitwise run to run
    again = fgmres(mv, b, jacobi, rtol=rtol, restart=restart, maxiter=maxiter)
    assert torch.equal(got.x, again.x) and got.residual_norm == again.residual_norm


def test_device_fgmres_basis_is_orthonormal():
    """After one cycle without preconditioner the stored basis V[0..k] is orthonormal."""
    from aquaflux_gb300.solve import KrylovWorkspace, fgmres

    a, b = _system(500, 3, spread=1.0)
    ws = KrylovWorkspace(500, 12)
    res = fgmres(lambda v: a @ v, b, rtol=1e-30, restart=12, maxiter=12, workspace=ws)
    assert res.iterations == 12 and not res.converged
    V = ws.V[:13]
    gram = V @ V.T
    assert torch.allclose(gram, torch.eye(13, dtype=torch.float64, device="cuda"), atol=1e-13)


def test_device_fgmres_stops_at_a_breakdown():
    """b in a 3-dimensional invariant subspace: the basis breaks down after three columns."""
    from aquaflux_gb300.solve import fgmres

    n = 12
    a = torch.zeros(n, n, dtype=torch.float64, device="cuda")
    a[:3, :3] = torch.tensor([[2.0, 1.0, 0.0], [0.0, 3.0, 1.0], [1.0, 0.0, 4.0]])
    a[3:, 3:] = torch.eye(n - 3) * 5.0
    b = torch.zeros(n, dtype=torch.float64, device="cuda")
    b[:3] = torch.tensor([1.0, -2.0, 0.5])
    q = fgmres(lambda v: a @ v, b, rtol=1e-14, restart=10, maxiter=20)
    assert q.converged and q.iterations == 3
    assert float(torch.linalg.vector_norm(a @ q.x - b)) <= 1e-12


def test_breakdown_keeps_the_queued_iteration_finite():
    """An exact breakdown on the first column (identity operator): the iteration queued behind it
    sees finite values, so a preconditioner that refuses non-finite input never fires."""
    from aquaflux_gb300.solve import fgmres

    b = torch.arange(1.0, 9.0, dtype=torch.float64, device="cuda")

    def strict(v):
        assert bool(torch.isfinite(v).all()), "preconditioner saw a non-finite vector"
        return v.clone()

    q = fgmres(lambda v: v.clone(), b, strict, rtol=1e-14, restart=5, maxiter=10)
    assert q.converged and q.iterations == 1
    assert torch.allclose(q.x, b, rtol=1e-15, atol=0.0)


def test_fgmres_refuses_host_tensors():
    from aquaflux_gb300.solve import fgmres

    with pytest.raises(ValueError):
        fgmres(lambda v: v, torch.ones(4, dtype=torch.float64))
