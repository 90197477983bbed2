"""The shifted, equilibrated cell-major operator restatement against the reference's outputs."""
import numpy as np

from oracle import operator_oracle as oo
from tests.cases import golden


def test_shift_equilibrate_matches_reference_bitwise():
    d = golden("operator")
    blocks, scale = oo.shift_equilibrate(d["op_blocks"], d["op_bsr_indptr"], d["op_bsr_indices"],
                                         d["op_shift"])
    data = oo.bsr_to_cell_major_csr_data(blocks, d["op_bsr_indptr"], d["op_bsr_indices"])
    assert np.array_equal(data, d["op_cm_data"])
    assert np.array_equal(scale, d["op_scale"])


def test_equilibrate_only_matches_reference_bitwise():
    d = golden("operator")
    blocks, scale = oo.shift_equilibrate(d["op_blocks"], d["op_bsr_indptr"], d["op_bsr_indices"])
    data = oo.bsr_to_cell_major_csr_data(blocks, d["op_bsr_indptr"], d["op_bsr_indices"])
    assert np.array_equal(data, d["op_eq_cm_data"])
    assert np.array_equal(scale, d["op_eq_scale"])


def test_cell_major_permutation_matches_reference():
    d = golden("operator")
    n, b = len(d["op_bsr_indptr"]) - 1, d["op_blocks"].shape[1]
    i, f = np.meshgrid(np.arange(n), np.arange(b), indexing="ij")
    assert np.array_equal((f * n + i).reshape(-1), d["op_perm"])


def test_shift_only_matches_reference_shifted_jacobian():
    """shifted_jacobian (sparse_jacobian.py:893-927): the same values in the field-major CSR."""
    d = golden("operator")
    blocks, _ = oo.shift_equilibrate(d["op_blocks"], d["op_bsr_indptr"], d["op_bsr_indices"],
                                     d["op_shift"], equilibrate=False)
    ip, ix = d["op_bsr_indptr"], d["op_bsr_indices"]
    n, b = len(ip) - 1, blocks.shape[1]
    rows = np.repeat(np.arange(n), np.diff(ip))
    r = (np.arange(b)[None, :, None] * n + rows[:, None, None]) * np.ones((1, 1, b), dtype=np.int64)
    c = (np.arange(b)[None, None, :] * n + ix[:, None, None]) * np.ones((1, b, 1), dtype=np.int64)
    order = np.argsort(r.ravel() * (n * b) + c.ravel())
    assert np.array_equal(blocks.ravel()[order], d["op_shifted_fm_data"])
