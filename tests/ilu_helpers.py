"""ctypes access to the CPU ILU(0) checker (the C restatement of the reference's kernel)."""
from __future__ import annotations

import ctypes
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def c_oracle():
    path = os.path.join(ROOT, "oracle", "libilu0_oracle.so")
    if not os.path.exists(path):
        import subprocess
        import sys

        subprocess.run([sys.executable, os.path.join(ROOT, "oracle", "build_oracle.py")], check=True)
    return ctypes.CDLL(path)


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def oracle_factor_solve(indptr, indices, values, rhs):
    """(diag, factor, solve, solve_transpose) from the C oracle; raises like the reference."""
    L = c_oracle()
    n = len(indptr) - 1
    ip = np.ascontiguousarray(indptr, dtype=np.int32)
    ix = np.ascontiguousarray(indices, dtype=np.int32)
    diag = np.zeros(n, dtype=np.int32)
    bad = ctypes.c_int(-1)
    rc = L.ilu0_diagonal_positions(_p(ip), _p(ix), n, _p(diag), ctypes.byref(bad))
    if rc == 3:
        raise ValueError(f"row {bad.value} stores no diagonal entry")
    data = np.array(values, dtype=np.float64)
    rc = L.ilu0_factor(_p(ip), _p(ix), _p(data), _p(diag), n, ctypes.byref(bad))
    if rc == 4:
        raise ZeroDivisionError(f"ILU(0) met an exactly zero pivot at row {bad.value}")
    x = np.array(rhs, dtype=np.float64)
    L.ilu0_solve(_p(ip), _p(ix), _p(data), _p(diag), _p(x), n)
    xt = np.array(rhs, dtype=np.float64)
    L.ilu0_solve_transpose(_p(ip), _p(ix), _p(data), _p(diag), _p(xt), n)
    return diag, data, x, xt


def cell_major(indptr, indices, values, n_cells, n_fields):
    """Permute a field-major operator to the cell-major interleaved order (cell * nf + field)."""
    import scipy.sparse as sp

    n = n_cells * n_fields
    a = sp.csr_matrix((values, indices, indptr), shape=(n, n))
    old = np.arange(n)
    new = (old % n_cells) * n_fields + old // n_cells
    perm = np.empty(n, dtype=np.int64)
    perm[new] = old
    b = a[perm][:, perm].tocsr()
    b.sort_indices()
    return b.indptr.astype(np.int32), b.indices.astype(np.int32), b.data.astype(np.float64)


def to_bsr(indptr, indices, values, b):
    """Scalar CSR with block-dense b x b structure -> BSR (row-major blocks)."""
    import scipy.sparse as sp

    n = len(indptr) - 1
    a = sp.csr_matrix((values, indices, indptr), shape=(n, n)).tobsr(blocksize=(b, b))
    a.sort_indices()
    return a.indptr.astype(np.int32), a.indices.astype(np.int32), a.data.reshape(-1).astype(np.float64)


def reference_kernel():
    """The reference's own compiled ILU(0) module (``oracle/build_ref.py``), or None where it is
    not built (no reference checkout or generated C on this machine)."""
    import sys

    sys.path.insert(0, ROOT)
    from oracle.build_ref import build_ref, load_ref

    try:
        build_ref()
    except RuntimeError:
        return None
    return load_ref()


def reference_factor_solve(mod, indptr, indices, values, rhs):
    """(diag, factor, solve, solve_transpose) from the reference's compiled kernel."""
    ip = np.ascontiguousarray(indptr, dtype=np.int32)
    ix = np.ascontiguousarray(indices, dtype=np.int32)
    n = len(ip) - 1
    diag = np.asarray(mod.diagonal_positions(ip, ix, n))
    data = np.array(values, dtype=np.float64)
    mod.factor(ip, ix, data, diag, n)
    x = np.array(rhs, dtype=np.float64)
    mod.solve(ip, ix, data, diag, x, n)
    xt = np.array(rhs, dtype=np.float64)
    mod.solve_transpose(ip, ix, data, diag, xt, n)
    return diag, data, x, xt


def random_block_operator(n_cells, b, seed):
    """A diagonally dominant cell-major operator on a 3D-grid-like block pattern (scalar CSR)."""
    import scipy.sparse as sp

    rng = np.random.default_rng(seed)
    n = n_cells
    side = max(2, round(n ** (1 / 3)))
    rows, cols = [np.arange(n)], [np.arange(n)]
    for off in (1, side, side * side):
        i = np.arange(n - off)
        rows += [i, i + off]
        cols += [i + off, i]
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    blocks = rng.standard_normal((r.size, b, b))
    blocks[r == c] += np.eye(b) * 4.0 * b
    coo_r = (r[:, None, None] * b + np.arange(b)[None, :, None]).repeat(b, 2).reshape(-1)
    coo_c = (c[:, None, None] * b + np.arange(b)[None, None, :]).repeat(b, 1).reshape(-1)
    A = sp.csr_matrix((blocks.reshape(-1), (coo_r, coo_c)), shape=(n * b, n * b))
    A.sort_indices()
    return A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data.astype(np.float64)
