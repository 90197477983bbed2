"""Block-stencil colouring bit-identical to the reference's (its own output, ``colouring.npz``)."""
from __future__ import annotations

import numpy as np
import pytest

from aquaflux_gb300.colouring import block_stencil_colouring, stencil_pattern
from tests.cases import golden


@pytest.mark.parametrize("name", ["c2d", "c3d", "c3p"])
@pytest.mark.parametrize("reach", [1, 2, 3])
def test_colouring_matches_reference(name, reach):
    d = golden("colouring")
    col = block_stencil_colouring(d[f"{name}_owner"], d[f"{name}_nb"], int(d[f"{name}_n"]), reach)
    np.testing.assert_array_equal(col.colour, d[f"{name}_r{reach}_colour"])
    np.testing.assert_array_equal(col.pattern_rows, d[f"{name}_r{reach}_rows"])
    np.testing.assert_array_equal(col.pattern_cols, d[f"{name}_r{reach}_cols"])


@pytest.mark.parametrize("reach", [1, 2])
def test_colouring_is_collision_free(reach):
    """Columns sharing a row of the pattern never share a colour (test_sparse_jacobian.py:50)."""
    d = golden("colouring")
    o, nb, n = d["c3p_owner"], d["c3p_nb"], int(d["c3p_n"])
    col = block_stencil_colouring(o, nb, n, reach)
    pat = stencil_pattern(o, nb, n, reach).tocsr()
    for r in range(n):
        cs = pat.indices[pat.indptr[r]:pat.indptr[r + 1]]
        assert len(set(col.colour[cs].tolist())) == cs.size


def test_reach_must_be_positive():
    d = golden("colouring")
    with pytest.raises(ValueError):
        block_stencil_colouring(d["c2d_owner"], d["c2d_nb"], int(d["c2d_n"]), 0)
