"""The host-side transpose map of a BSR pattern (``fv_bsr_transpose_map``, no GPU): for every block
row j of A^T the rows i of A holding a block (i, j), ascending, and that block's index in A --
checked against scipy's transpose; malformed patterns are refused."""
from __future__ import annotations

import numpy as np
import pytest
import scipy.sparse as sp

from aquaflux_gb300._lib import FvError, check, lib, ptr


def _map(ip, ix):
    n = len(ip) - 1
    tp, ti, tb = (np.empty(k, dtype=np.int32) for k in (n + 1, int(ip[-1]), int(ip[-1])))
    check(lib().fv_bsr_transpose_map(n, ptr(ip), ptr(ix), ptr(tp), ptr(ti), ptr(tb)))
    return tp, ti, tb


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_transpose_map_is_the_pattern_transpose(seed):
    n = 200
    a = (sp.random(n, n, density=0.03, random_state=seed, format="csr") + sp.eye(n)).tocsr()
    a.sort_indices()
    ip, ix = a.indptr.astype(np.int32), a.indices.astype(np.int32)
    tp, ti, tb = _map(ip, ix)
    # scipy's transpose with the block numbers as data
    t = sp.csr_matrix((np.arange(ix.size) + 1.0, ix, ip), shape=(n, n)).T.tocsr()
    t.sort_indices()
    assert np.array_equal(tp, t.indptr) and np.array_equal(ti, t.indices)
    assert np.array_equal(tb, t.data.astype(np.int64) - 1)
    rows = np.repeat(np.arange(n), np.diff(ip))
    assert np.array_equal(rows[tb], ti) and np.array_equal(ix[tb], np.repeat(np.arange(n), np.diff(tp)))


def test_transpose_map_refuses_malformed_patterns():
    ip = np.array([0, 2, 1, 3], dtype=np.int32)  # decreasing
    ix = np.array([0, 1, 2], dtype=np.int32)
    with pytest.raises(FvError, match="non-decreasing"):
        _map(ip, ix)
    ip = np.array([0, 1, 2, 3], dtype=np.int32)
    ix = np.array([0, 3, 2], dtype=np.int32)  # column 3 of a 3 x 3 pattern
    with pytest.raises(FvError, match="out of range"):
        _map(ip, ix)
