"""Host half of bench.py's ILU(0) CPU-vs-GPU baseline (no GPU): the BSR -> cell-major scalar CSR
conversion, and the timed C restatement giving the same factor and solution as the oracle."""
import numpy as np
import scipy.sparse as sp

import bench
from tests.ilu_helpers import oracle_factor_solve


def _random_bsr(n, b, seed):
    rng = np.random.default_rng(seed)
    a = sp.random(n, n, density=0.08, random_state=seed, format="csr") + sp.eye(n)
    a = ((a + a.T) > 0).astype(np.float64).tocsr()
    a.sort_indices()
    ip, ix = a.indptr.astype(np.int32), a.indices.astype(np.int32)
    blocks = rng.standard_normal((ix.size, b, b))
    rows = np.repeat(np.arange(n), np.diff(ip))
    blocks[rows == ix] += 8.0 * np.eye(b)  # dominant diagonal blocks
    return ip, ix, blocks


def test_bsr_to_scalar_csr_is_the_same_operator_in_cell_major_rows():
    ip, ix, blocks = _random_bsr(40, 3, 0)
    sptr, scols, sdata = bench.bsr_to_scalar_csr(blocks, ip, ix)
    want = sp.bsr_matrix((blocks, ix, ip), shape=(120, 120)).tocsr()
    want.sort_indices()
    assert np.array_equal(sptr, want.indptr) and np.array_equal(scols, want.indices)
    assert np.array_equal(sdata, want.data)


def test_timed_c_ilu0_equals_the_oracle():
    ip, ix, blocks = _random_bsr(60, 4, 1)
    sptr, scols, sdata = bench.bsr_to_scalar_csr(blocks, ip, ix)
    rhs = np.random.default_rng(2).standard_normal(sptr.size - 1)
    got = bench.cpu_ilu0(sptr, scols, sdata, rhs)
    _, factor, x, _ = oracle_factor_solve(sptr, scols, sdata, rhs)
    assert np.array_equal(got["factor"], factor) and np.array_equal(got["x"], x)
    assert got["factor_s"] >= 0.0 and got["solve_s"] >= 0.0
