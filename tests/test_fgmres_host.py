"""FGMRES on CPU tensors (no GPU): the lagged variant (convergence test one iteration behind,
columns read back after the next iteration is queued) reproduces the plain one, across restarts,
early convergence, the iteration cap and a breakdown."""
import numpy as np
import pytest
import torch

from aquaflux_gb300.solve import fgmres


def _system(n, seed):
    rng = np.random.default_rng(seed)
    a = np.eye(n) * 4.0 + rng.standard_normal((n, n)) / np.sqrt(n)
    a[np.tril_indices(n, -3)] *= 0.1
    return torch.tensor(a), torch.tensor(rng.standard_normal(n))


@pytest.mark.parametrize("restart,maxiter,rtol", [(30, 300, 1e-10), (5, 300, 1e-10),
                                                  (30, 300, 1e-3), (4, 9, 1e-12)])
def test_lagged_fgmres_equals_plain(restart, maxiter, rtol):
    a, b = _system(60, 0)
    d = torch.diagonal(a).clone()
    calls = {"plain": 0, "lag": 0}

    def mv(key):
        def f(v):
            calls[key] += 1
            return a @ v
        return f

    def jacobi(v):
        return v / d

    p = fgmres(mv("plain"), b, jacobi, rtol=rtol, restart=restart, maxiter=maxiter)
    q = fgmres(mv("lag"), b, jacobi, rtol=rtol, restart=restart, maxiter=maxiter, lag=True)
    assert torch.equal(p.x, q.x)
    assert (p.iterations, p.converged, p.residual_norm) == (q.iterations, q.converged,
                                                            q.residual_norm)
    # the lagged run queues at most one discarded iteration per restart cycle
    cycles = -(-p.iterations // restart) + 1
    assert calls["plain"] <= calls["lag"] <= calls["plain"] + cycles


def test_lagged_fgmres_stops_at_a_breakdown():
    """b in a 3-dimensional invariant subspace: the basis breaks down after three columns (a zero
    norm), which both variants take as the exact solution."""
    n = 12
    a = torch.zeros(n, n, dtype=torch.float64)
    a[:3, :3] = torch.tensor([[2.0, 1.0, 0.0], [0.0, 3.0, 1.0], [1.0, 0.0, 4.0]])
    a[3:, 3:] = torch.eye(n - 3) * 5.0
    b = torch.zeros(n, dtype=torch.float64)
    b[:3] = torch.tensor([1.0, -2.0, 0.5])
    p = fgmres(lambda v: a @ v, b, rtol=1e-14, restart=10, maxiter=20)
    q = fgmres(lambda v: a @ v, b, rtol=1e-14, restart=10, maxiter=20, lag=True)
    assert p.converged and q.converged and p.iterations == q.iterations == 3
    assert torch.equal(p.x, q.x)
    assert float(torch.linalg.vector_norm(a @ q.x - b)) <= 1e-12


def test_lagged_fgmres_breakdown_keeps_the_queued_iteration_finite():
    """An exact breakdown on the first column (identity operator): the iteration queued behind it
    must see finite values, so a preconditioner that refuses non-finite input never fires."""
    n = 8
    b = torch.arange(1.0, n + 1.0, dtype=torch.float64)

    def strict(v):
        assert torch.isfinite(v).all(), "preconditioner saw a non-finite vector"
        return v

    q = fgmres(lambda v: v.clone(), b, strict, rtol=1e-14, restart=5, maxiter=10, lag=True)
    assert q.converged and q.iterations == 1
    assert torch.equal(q.x, b)
