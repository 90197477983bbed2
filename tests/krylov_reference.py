"""Flexible GMRES(m) in plain torch (any device) -- test infrastructure only, the checker of the
device FGMRES in ``aquaflux_gb300.solve.fgmres``.

Right-preconditioned, restarted, CGS2 orthogonalisation, Givens rotations on the host, the
residual estimate ``|g_{j+1}|`` as the stopping test and the true residual at the end of every
cycle: the method of lineax GMRES behind the reference's ``solve_linear``
(``aquaflux/solve/linear.py:199-298``), written out step by step.
"""
from __future__ import annotations

import math

import numpy as np
import torch


def fgmres_reference(matvec, b, precond=None, *, rtol=1e-3, atol=0.0, restart=30, maxiter=300):
    """``(x, iterations, residual_norm, converged)``."""
    M = precond if precond is not None else (lambda v: v)
    x = torch.zeros_like(b)
    bnorm = float(torch.linalg.vector_norm(b))
    tol = max(atol, rtol * bnorm)
    r, beta, total = b.clone(), bnorm, 0
    if beta <= tol:
        return x, 0, beta, True
    while total < maxiter:
        m = min(restart, maxiter - total)
        V = torch.empty(m + 1, b.numel(), dtype=b.dtype, device=b.device)
        Z = torch.empty(m, b.numel(), dtype=b.dtype, device=b.device)
        H = np.zeros((m + 1, m))
        cs, sn, g = np.zeros(m), np.zeros(m), np.zeros(m + 1)
        g[0] = beta
        V[0] = r / beta
        k = 0
        for j in range(m):
            Z[j] = M(V[j])
            w = matvec(Z[j])
            Vj = V[: j + 1]
            h1 = Vj @ w
            w = w - h1 @ Vj
            h2 = Vj @ w
            w = w - h2 @ Vj
            hn = float(torch.linalg.vector_norm(w))
            H[: j + 1, j] = (h1 + h2).cpu().numpy()
            H[j + 1, j] = hn
            if hn > 0:
                V[j + 1] = w / hn
            for i in range(j):
                t = cs[i] * H[i, j] + sn[i] * H[i + 1, j]
                H[i + 1, j] = -sn[i] * H[i, j] + cs[i] * H[i + 1, j]
                H[i, j] = t
            den = math.hypot(H[j, j], H[j + 1, j])
            cs[j], sn[j] = (1.0, 0.0) if den == 0 else (H[j, j] / den, H[j + 1, j] / den)
            H[j, j] = cs[j] * H[j, j] + sn[j] * H[j + 1, j]
            H[j + 1, j] = 0.0
            g[j + 1] = -sn[j] * g[j]
            g[j] = cs[j] * g[j]
            k, total = j + 1, total + 1
            if abs(g[j + 1]) <= tol or hn == 0:
                break
        y = np.zeros(k)
        for i in range(k - 1, -1, -1):
            y[i] = (g[i] - H[i, i + 1:k] @ y[i + 1:]) / H[i, i]
        x = x + torch.as_tensor(y, dtype=b.dtype, device=b.device) @ Z[:k]
        r = b - matvec(x)
        beta = float(torch.linalg.vector_norm(r))
        if beta <= tol:
            return x, total, beta, True
    return x, total, beta, False
