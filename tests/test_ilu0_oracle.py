"""The C restatement of ILU(0) against the reference's Python twin's golden vectors, and bit for
bit against the reference's own compiled kernel (``aquaflux/solve/_ilu0.pyx``, built from its
source by ``oracle/build_ref.py``; skipped where it cannot be built)."""
from __future__ import annotations

import numpy as np
import pytest

from tests.cases import golden
from tests.ilu_helpers import (oracle_factor_solve, random_block_operator, reference_factor_solve,
                               reference_kernel)


def test_c_oracle_matches_reference_twin_bitwise():
    d = golden("ilu0")
    diag, data, x, xt = oracle_factor_solve(d["ilu_indptr"], d["ilu_indices"], d["ilu_values"],
                                            d["ilu_rhs"])
    np.testing.assert_array_equal(diag, d["ilu_diag"])
    # the reference twin uses numpy dot / subtract.at, whose rounding may differ from the
    # sequential kernel by an ulp -- pinned to 1e-13 here and bitwise to the compiled kernel below
    np.testing.assert_allclose(data, d["ilu_factor"], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(x, d["ilu_solve"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(xt, d["ilu_solve_t"], rtol=1e-12, atol=1e-14)


def test_errors_match_reference_semantics():
    ip = np.array([0, 1, 2], dtype=np.int32)
    ix = np.array([0, 0], dtype=np.int32)  # row 1 has no diagonal
    with pytest.raises(ValueError, match="row 1"):
        oracle_factor_solve(ip, ix, np.array([1.0, 2.0]), np.zeros(2))
    ip = np.array([0, 2, 4], dtype=np.int32)
    ix = np.array([0, 1, 0, 1], dtype=np.int32)
    with pytest.raises(ZeroDivisionError, match="row 0"):
        oracle_factor_solve(ip, ix, np.array([0.0, 1.0, 1.0, 1.0]), np.zeros(2))


@pytest.mark.parametrize("case", ["fixture", "block6"])
def test_c_oracle_matches_the_reference_kernel_bitwise(case):
    mod = reference_kernel()
    if mod is None:
        pytest.skip("the reference's compiled ILU(0) is not built on this machine")
    if case == "fixture":
        d = golden("ilu0")
        ip, ix, vals, rhs = d["ilu_indptr"], d["ilu_indices"], d["ilu_values"], d["ilu_rhs"]
    else:
        ip, ix, vals = random_block_operator(343, 6, seed=3)
        rhs = np.random.default_rng(4).standard_normal(len(ip) - 1)
    want = reference_factor_solve(mod, ip, ix, vals, rhs)
    got = oracle_factor_solve(ip, ix, vals, rhs)
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)


def test_reference_kernel_errors():
    mod = reference_kernel()
    if mod is None:
        pytest.skip("the reference's compiled ILU(0) is not built on this machine")
    ip = np.array([0, 1, 2], dtype=np.int32)
    ix = np.array([0, 0], dtype=np.int32)
    with pytest.raises(ValueError, match="row 1"):
        mod.diagonal_positions(ip, ix, 2)
