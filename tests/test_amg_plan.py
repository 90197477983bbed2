"""Host plan of the aggregation hierarchy (no GPU): aggregates partition the cells, the ordered
fine-block lists reproduce the Galerkin product P^T A P of the piecewise-constant prolongation,
and colour-ordered coarse levels have shallow ILU(0) level schedules."""
import numpy as np
import pytest
import scipy.sparse as sp

from aquaflux_gb300 import workloads
from aquaflux_gb300.amg import plan_hierarchy


def _cell_graph(n_ax):
    m = workloads.channel3d(n_ax, renumber="host").mesh
    o, nb = np.asarray(m.owner), np.asarray(m.neighbour)
    keep = nb >= 0
    n = m.n_cells
    a = sp.coo_matrix((np.ones(int(keep.sum())), (o[keep], nb[keep])), shape=(n, n))
    a = (a + a.T + sp.eye(n)).tocsr()
    a.sort_indices()
    return n, a.indptr.astype(np.int32), a.indices.astype(np.int32)


def _lower_depth(ip, ix):
    n = len(ip) - 1
    lev = np.zeros(n, np.int64)
    for i in range(n):
        lo = ix[ip[i]:ip[i + 1]]
        lo = lo[lo < i]
        if lo.size:
            lev[i] = lev[lo].max() + 1
    return int(lev.max()) + 1


@pytest.mark.parametrize("order", ["colour", "natural"])
def test_plan_partitions_cells_and_forms_galerkin_blocks(order):
    n, ip, ix = _cell_graph(12)
    plan = plan_hierarchy(n, ip, ix, min_cells=50, coarse_order=order)
    assert len(plan) >= 2
    rng = np.random.default_rng(0)
    b = 2
    vals = rng.standard_normal((int(ip[-1]), b, b))
    for step in plan:
        na, agg = step["n_coarse"], step["agg"]
        assert agg.min() == 0 and agg.max() == na - 1 and np.unique(agg).size == na
        assert np.array_equal(np.sort(step["mlist"]), np.arange(len(agg)))
        for i in range(na):
            assert np.all(agg[step["mlist"][step["mptr"][i]:step["mptr"][i + 1]]] == i)
        # coarse blocks from the ordered fine-block lists == P^T A P
        gp, gl = step["gptr"], step["glist"]
        coarse = np.stack([vals[gl[gp[q]:gp[q + 1]]].sum(axis=0) for q in range(len(gp) - 1)])
        A = sp.bsr_matrix((vals, ix, ip), shape=(len(agg) * b, len(agg) * b)).toarray()
        P = np.zeros((len(agg) * b, na * b))
        for i, g in enumerate(agg):
            P[i * b:(i + 1) * b, g * b:(g + 1) * b] = np.eye(b)
        cip, cix = step["indptr"], step["indices"]
        C = sp.bsr_matrix((coarse, cix, cip), shape=(na * b, na * b)).toarray()
        np.testing.assert_allclose(C, P.T @ A @ P, rtol=1e-12, atol=1e-12)
        for i in range(na):
            row = cix[cip[i]:cip[i + 1]]
            assert np.all(np.diff(row) > 0) and i in row
        vals, ip, ix = coarse, cip, cix


def test_colour_order_gives_shallow_coarse_level_sets():
    n, ip, ix = _cell_graph(16)
    nat = plan_hierarchy(n, ip, ix, min_cells=200, coarse_order="natural")
    col = plan_hierarchy(n, ip, ix, min_cells=200, coarse_order="colour")
    d_nat = _lower_depth(nat[0]["indptr"], nat[0]["indices"])
    d_col = _lower_depth(col[0]["indptr"], col[0]["indices"])
    assert d_col <= 16 < d_nat


def test_aggregate_colouring_is_saturation_colouring_of_the_coarse_pattern():
    """The coarse-level colouring read from the fine pattern gives the same colours as the
    saturation colouring of the coarse pattern formed by a full coarsening step."""
    import ctypes

    from aquaflux_gb300._lib import check, lib, ptr
    from aquaflux_gb300.amg import _coarsen

    n, ip, ix = _cell_graph(14)
    agg = np.empty(n, np.int32)
    na = ctypes.c_int(0)
    check(lib().fv_aggregate(n, ptr(ip), ptr(ix), ptr(agg), ctypes.byref(na)))
    na = na.value
    got, nc_got = np.empty(na, np.int32), ctypes.c_int(0)
    check(lib().fv_colour_aggregates(n, ptr(ip), ptr(ix), ptr(agg), na, ptr(got),
                                     ctypes.byref(nc_got)))
    step = _coarsen(n, ip, ix, agg, na, lists=False)
    want, nc_want = np.empty(na, np.int32), ctypes.c_int(0)
    check(lib().fv_saturation_colouring(na, ptr(step["indptr"]), ptr(step["indices"]), ptr(want),
                                        ctypes.byref(nc_want)))
    assert np.array_equal(got, want) and nc_got.value == nc_want.value
    cip, cix = step["indptr"], step["indices"]
    for a in range(na):  # a proper colouring of the aggregate graph
        nb = cix[cip[a]:cip[a + 1]]
        assert np.all(got[nb[nb != a]] != got[a])


def test_cell_pattern_equals_the_reach_one_stencil():
    from aquaflux_gb300.colouring import cell_pattern, stencil_pattern

    m = workloads.channel3d(10, renumber="host").mesh
    o, nb = np.asarray(m.owner), np.asarray(m.neighbour)
    keep = nb >= 0
    ip, ix = cell_pattern(o[keep], nb[keep], m.n_cells)
    ref = stencil_pattern(o[keep], nb[keep], m.n_cells, 1).tocsr()
    ref.sort_indices()
    assert np.array_equal(ip, ref.indptr) and np.array_equal(ix, ref.indices)


def test_permuted_pattern_maps_every_block():
    """fv_permute_pattern: new block (r, c) is old block (perm[r], perm[c])."""
    import ctypes

    from aquaflux_gb300._lib import check, lib, ptr

    n, ip, ix = _cell_graph(6)
    perm = np.random.default_rng(1).permutation(n).astype(np.int32)
    pip = np.empty(n + 1, np.int32)
    pix = np.empty(ip[-1], np.int32)
    bmap = np.empty(ip[-1], np.int64)
    check(lib().fv_permute_pattern(n, ptr(ip), ptr(ix), ptr(perm), ptr(pip), ptr(pix), ptr(bmap)))
    rows_old = np.repeat(np.arange(n), np.diff(ip))
    rows_new = np.repeat(np.arange(n), np.diff(pip))
    assert np.array_equal(perm[rows_new], rows_old[bmap])
    assert np.array_equal(perm[pix], ix[bmap])
    assert np.array_equal(np.sort(bmap), np.arange(ip[-1]))
    for r in range(n):
        assert np.all(np.diff(pix[pip[r]:pip[r + 1]]) > 0)
    bad = perm.copy()
    bad[0] = bad[1]
    with pytest.raises(Exception):
        check(lib().fv_permute_pattern(n, ptr(ip), ptr(ix), ptr(bad), ptr(pip), ptr(pix),
                                       ptr(bmap)))


def test_host_passes_reject_out_of_range_indices():
    """The pattern passes check their column indices (over the host threads) and report the
    error instead of reading out of bounds: coarsening, aggregate colouring, permutation and the
    cell pattern."""
    import ctypes

    from aquaflux_gb300._lib import FvError, check, lib, ptr

    n, ip, ix = _cell_graph(6)
    agg = np.empty(n, np.int32)
    na = ctypes.c_int(0)
    check(lib().fv_aggregate(n, ptr(ip), ptr(ix), ptr(agg), ctypes.byref(na)))
    na = na.value
    bad = ix.copy()
    bad[len(bad) // 2] = n  # one column past the last cell
    nnz = int(ip[-1])
    col, nco = np.empty(na, np.int32), ctypes.c_int(0)
    with pytest.raises(FvError, match="column index out of range"):
        check(lib().fv_colour_aggregates(n, ptr(ip), ptr(bad), ptr(agg), na, ptr(col),
                                         ctypes.byref(nco)))
    mptr, mlist = np.empty(na + 1, np.int32), np.empty(n, np.int32)
    cip, cix = np.empty(na + 1, np.int32), np.empty(nnz, np.int32)
    gptr, glist, ncb = np.empty(nnz + 1, np.int64), np.empty(nnz, np.int64), ctypes.c_long(0)
    with pytest.raises(FvError, match="column index out of range"):
        check(lib().fv_coarsen(n, ptr(ip), ptr(bad), ptr(agg), na, ptr(mptr), ptr(mlist),
                               ptr(cip), ptr(cix), ptr(gptr), ptr(glist), ctypes.byref(ncb)))
    perm = np.arange(n, dtype=np.int32)
    pip, pix, bmap = np.empty(n + 1, np.int32), np.empty(nnz, np.int32), np.empty(nnz, np.int64)
    with pytest.raises(FvError, match="column index out of range"):
        check(lib().fv_permute_pattern(n, ptr(ip), ptr(bad), ptr(perm), ptr(pip), ptr(pix),
                                       ptr(bmap)))
    owner = np.array([0, 1, 2], np.int32)
    neigh = np.array([1, 2, n], np.int32)
    cp_ip, cp_ix = np.empty(n + 1, np.int32), np.empty(n + 6, np.int32)
    with pytest.raises(FvError, match="out of range at pair 2"):
        check(lib().fv_cell_pattern(n, 3, ptr(owner), ptr(neigh), ptr(cp_ip), ptr(cp_ix)))


def test_host_graph_routines_refuse_a_decreasing_offset_list():
    """Every host routine that walks a CSR pattern checks its offsets first (a decreasing indptr
    would make it read past the index array): aggregation, aggregate colouring, coarsening,
    permutation, both colourings and the transpose map."""
    import ctypes

    from aquaflux_gb300._lib import FvError, check, lib, ptr

    n, ip, ix = _cell_graph(6)
    agg = np.zeros(n, np.int32)
    na = ctypes.c_int(0)
    check(lib().fv_aggregate(n, ptr(ip), ptr(ix), ptr(agg), ctypes.byref(na)))
    na = na.value
    bad = ip.copy()
    bad[n // 2] = bad[n // 2 + 1] + 1  # one row "ends" before it starts
    nnz = int(ip[-1])
    i32 = lambda k: np.empty(k, np.int32)  # noqa: E731
    i64 = lambda k: np.empty(k, np.int64)  # noqa: E731
    calls = {
        "fv_aggregate": lambda: lib().fv_aggregate(n, ptr(bad), ptr(ix), ptr(i32(n)),
                                                   ctypes.byref(ctypes.c_int(0))),
        "fv_colour_aggregates": lambda: lib().fv_colour_aggregates(
            n, ptr(bad), ptr(ix), ptr(agg), na, ptr(i32(na)), ctypes.byref(ctypes.c_int(0))),
        "fv_coarsen": lambda: lib().fv_coarsen(
            n, ptr(bad), ptr(ix), ptr(agg), na, ptr(i32(na + 1)), ptr(i32(n)), ptr(i32(na + 1)),
            ptr(i32(nnz)), ptr(i64(nnz + 1)), ptr(i64(nnz)), ctypes.byref(ctypes.c_long(0))),
        "fv_permute_pattern": lambda: lib().fv_permute_pattern(
            n, ptr(bad), ptr(ix), ptr(np.arange(n, dtype=np.int32)), ptr(i32(n + 1)),
            ptr(i32(nnz)), ptr(i64(nnz))),
        "fv_saturation_colouring": lambda: lib().fv_saturation_colouring(
            n, ptr(bad), ptr(ix), ptr(i32(n)), ctypes.byref(ctypes.c_int(0))),
        "fv_greedy_colouring": lambda: lib().fv_greedy_colouring(
            n, ptr(bad), ptr(ix), ptr(i32(n)), ctypes.byref(ctypes.c_int(0))),
        "fv_bsr_transpose_map": lambda: lib().fv_bsr_transpose_map(
            n, ptr(bad), ptr(ix), ptr(i32(n + 1)), ptr(i32(nnz)), ptr(i32(nnz))),
    }
    for name, call in calls.items():
        with pytest.raises(FvError, match=name + ": indptr is not a non-decreasing"):
            check(call())
