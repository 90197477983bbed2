"""CPU restatement (numpy) of the shifted, equilibrated cell-major operator -- test
infrastructure only, the checker of ``fv_bsr_shift_equilibrate``.

``ShiftedCellMajorOperator.assemble`` (``aquaflux/solve/amg_preconditioner.py:545-658``): add the
pseudo-transient shift ``beta d`` (field-major) to the diagonal, take the symmetric square-root
equilibration ``s = 1 / sqrt(|diag|)`` (``|0|`` read as 1; ``frozen_operator.py:121-143``) and
scale every stored entry by ``s[row]`` then ``s[column]`` (``frozen_operator.py:72-118``), in the
cell-major order ``(cell i, field f) -> i * b + f`` (``ordering.py:52-77``).  Here the matrix is
held as cell-major BSR blocks, which is that order.  Pinned bitwise against the reference's own
outputs (``tests/golden/operator.npz``).
"""
from __future__ import annotations

import numpy as np


def shift_equilibrate(blocks, indptr, indices, shift_fm=None, equilibrate=True):
    """``(blocks', scale_fm)`` for BSR ``blocks`` (nnzb, b, b); ``scale_fm`` is None when not
    equilibrating."""
    blocks = np.array(blocks, dtype=np.float64, copy=True)
    n, b = len(indptr) - 1, blocks.shape[1]
    rows = np.repeat(np.arange(n), np.diff(indptr))
    dq = np.flatnonzero(rows == indices)
    if dq.size != n:
        raise ValueError("every block row needs its diagonal block")
    diag = blocks[dq][:, np.arange(b), np.arange(b)]  # (n, b) cell-major
    if shift_fm is not None:
        diag = diag + np.asarray(shift_fm, dtype=np.float64).reshape(b, n).T
        blocks[dq[:, None], np.arange(b)[None, :], np.arange(b)[None, :]] = diag
    if not equilibrate:
        return blocks, None
    mag = np.abs(diag)
    mag[mag == 0.0] = 1.0
    s = 1.0 / np.sqrt(mag)  # (n, b)
    blocks *= s[rows][:, :, None]
    blocks *= s[indices][:, None, :]
    return blocks, s.T.reshape(-1).copy()


def bsr_to_cell_major_csr_data(blocks, indptr, indices):
    """The data array of the cell-major scalar CSR with every block entry stored, rows sorted."""
    n, b = len(indptr) - 1, blocks.shape[1]
    out = []
    for i in range(n):
        q = np.arange(indptr[i], indptr[i + 1])
        for a in range(b):
            out.append(blocks[q, a, :].reshape(-1))
    return np.concatenate(out)
