"""CUDA BSR SpMV and ILU(0) against the CPU oracle (bitwise in fp64) and the reference fixture."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from tests.cases import golden
from tests.ilu_helpers import cell_major, oracle_factor_solve, to_bsr

pytestmark = pytest.mark.gpu


def _dev(a, dtype=None):
    t = torch.as_tensor(np.asarray(a))
    return t.to("cuda", dtype=dtype) if dtype is not None else t.to("cuda")


def test_scalar_ilu0_fp64_bitwise_equals_oracle():
    from aquaflux_gb300.ilu0 import Ilu0

    d = golden("ilu0")
    ip, ix, vals, rhs = d["ilu_indptr"], d["ilu_indices"], d["ilu_values"], d["ilu_rhs"]
    _, data, x, xt = oracle_factor_solve(ip, ix, vals, rhs)
    f = Ilu0.from_csr(ip, ix, vals, block_size=1, precision=64)
    np.testing.assert_array_equal(f.factor_values().cpu().numpy(), data)
    np.testing.assert_array_equal(f.solve(rhs).cpu().numpy(), x)
    np.testing.assert_array_equal(f.solve(rhs, transpose=True).cpu().numpy(), xt)


def test_block_ilu0_fp64_bitwise_equals_scalar_on_cell_major_order():
    from aquaflux_gb300.ilu0 import Ilu0

    d = golden("ilu0")
    ip, ix, vals = cell_major(d["ilu_indptr"], d["ilu_indices"], d["ilu_values"], 40, 3)
    rhs = d["ilu_rhs"]
    _, data, x, xt = oracle_factor_solve(ip, ix, vals, rhs)
    bp, bi, bv = to_bsr(ip, ix, vals, 3)
    f = Ilu0.from_csr(bp, bi, bv, block_size=3, precision=64)
    # the block factor, read back through the scalar pattern, equals the scalar factor
    sp_ip, sp_ix, sp_data = to_scalar(bp, bi, f.factor_values().cpu().numpy(), 3)
    np.testing.assert_array_equal(sp_ip, ip)
    np.testing.assert_array_equal(sp_ix, ix)
    np.testing.assert_array_equal(sp_data, data)
    # the transposed solve keeps the reference's operation order (bitwise); the block forward
    # solve subtracts off-diagonal blocks before in-block terms in its upper sweep and multiplies
    # by the pivots' reciprocals (1e-13)
    np.testing.assert_allclose(f.solve(rhs).cpu().numpy(), x, rtol=1e-13, atol=1e-15)
    np.testing.assert_array_equal(f.solve(rhs, transpose=True).cpu().numpy(), xt)


def to_scalar(bp, bi, bv, b):
    import scipy.sparse as sp

    n = (len(bp) - 1) * b
    a = sp.bsr_matrix((bv.reshape(-1, b, b), bi, bp), shape=(n, n)).tocsr()
    a.sort_indices()
    return a.indptr.astype(np.int32), a.indices.astype(np.int32), a.data


def test_fp32_ilu0_close_to_fp64():
    from aquaflux_gb300.ilu0 import Ilu0

    d = golden("ilu0")
    ip, ix, vals = cell_major(d["ilu_indptr"], d["ilu_indices"], d["ilu_values"], 40, 3)
    bp, bi, bv = to_bsr(ip, ix, vals, 3)
    f64 = Ilu0.from_csr(bp, bi, bv, block_size=3, precision=64)
    f32 = Ilu0.from_csr(bp, bi, bv, block_size=3, precision=32)
    rhs = d["ilu_rhs"]
    a = f64.solve(rhs).cpu().numpy()
    b = f32.solve(rhs).cpu().numpy()
    assert np.abs(a - b).max() <= 1e-5 * np.abs(a).max()


def test_transpose_identity():
    """<y, M r> = <M^T y, r> (tests/unit/test_ilu0.py:92-107)."""
    from aquaflux_gb300.ilu0 import Ilu0

    d = golden("ilu0")
    f = Ilu0.from_csr(d["ilu_indptr"], d["ilu_indices"], d["ilu_values"], block_size=1)
    rng = np.random.default_rng(1)
    y, r = rng.standard_normal((2, len(d["ilu_rhs"])))
    lhs = float(np.dot(y, f.solve(r).cpu().numpy()))
    rhs = float(np.dot(f.solve(y, transpose=True).cpu().numpy(), r))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_missing_diagonal_and_zero_pivot_raise_like_the_reference():
    from aquaflux_gb300.ilu0 import Ilu0

    with pytest.raises(ValueError, match="store no diagonal entry"):
        Ilu0.from_csr(np.array([0, 1, 2]), np.array([0, 0]), np.array([1.0, 2.0]), block_size=1)
    with pytest.raises(ZeroDivisionError, match="zero pivot at row 0"):
        Ilu0.from_csr(np.array([0, 2, 4]), np.array([0, 1, 0, 1]), np.array([0.0, 1.0, 1.0, 1.0]),
                      block_size=1)


@pytest.mark.parametrize("b", [1, 3, 6])
@pytest.mark.parametrize("transpose", [False, True])
def test_bsr_spmv_matches_scipy(b, transpose):
    import scipy.sparse as sp

    from aquaflux_gb300.sparse import bsr_spmv

    rng = np.random.default_rng(b)
    nb = 50
    a = sp.random(nb, nb, density=0.1, random_state=b, format="csr") + sp.eye(nb)
    a.sort_indices()
    vals = rng.standard_normal((a.nnz, b, b))
    dense = sp.bsr_matrix((vals, a.indices, a.indptr), shape=(nb * b, nb * b))
    x = rng.standard_normal(nb * b)
    want = (dense.T if transpose else dense) @ x
    got = bsr_spmv(a.indptr, a.indices, vals.reshape(-1), b, x, transpose=transpose)
    np.testing.assert_allclose(got.cpu().numpy(), want, rtol=1e-12, atol=1e-12)
    got32 = bsr_spmv(a.indptr, a.indices, vals.reshape(-1).astype(np.float32), b,
                     x.astype(np.float32), transpose=transpose)
    np.testing.assert_allclose(got32.cpu().numpy(), want, rtol=1e-4, atol=1e-4)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_transposed_spmv_block_size_kernels_agree_bitwise(dtype):
    """The transposed product's compile-time-size kernel (x 16-byte aligned) and its runtime-size
    kernel (x at an 8- or 4-byte offset) accumulate the same products in the same order."""
    import scipy.sparse as sp

    from aquaflux_gb300.sparse import bsr_spmv

    b, nb = 6, 400
    a = sp.random(nb, nb, density=0.02, random_state=3, format="csr") + sp.eye(nb)
    a.sort_indices()
    g = torch.Generator(device="cuda").manual_seed(3)
    vals = torch.randn(a.nnz * b * b, dtype=dtype, device="cuda", generator=g)
    buf = torch.randn(nb * b + 1, dtype=dtype, device="cuda", generator=g)
    x_off = buf[1:]
    x_al = x_off.clone()
    assert x_al.data_ptr() % 16 == 0 and x_off.data_ptr() % 16 != 0
    y_al = bsr_spmv(a.indptr, a.indices, vals, b, x_al, transpose=True)
    y_off = bsr_spmv(a.indptr, a.indices, vals, b, x_off, transpose=True)
    assert torch.equal(y_al, y_off)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_transposed_blocks_give_the_mapped_transposed_product_bitwise(dtype):
    """fv_bsr_transpose_blocks + the forward product on A^T's pattern (what the V-cycle's
    transposed products run) against fv_bsr_spmv_t_mapped: the same products, the same order."""
    import scipy.sparse as sp

    from aquaflux_gb300._lib import check, lib, ptr

    b, nb = 6, 300
    a = sp.random(nb, nb, density=0.03, random_state=8, format="csr") + sp.eye(nb)
    a.sort_indices()
    ip, ix = a.indptr.astype(np.int32), a.indices.astype(np.int32)
    nnzb = int(ip[-1])
    tp, ti, tb = (np.empty(n, dtype=np.int32) for n in (nb + 1, nnzb, nnzb))
    check(lib().fv_bsr_transpose_map(nb, ptr(ip), ptr(ix), ptr(tp), ptr(ti), ptr(tb)))
    tp, ti, tb = (torch.tensor(v, device="cuda") for v in (tp, ti, tb))
    g = torch.Generator(device="cuda").manual_seed(8)
    vals = torch.randn(nnzb * b * b, dtype=dtype, device="cuda", generator=g)
    x = torch.randn(nb * b, dtype=dtype, device="cuda", generator=g)
    f64 = int(dtype == torch.float64)
    st = torch.cuda.current_stream().cuda_stream
    want = torch.empty_like(x)
    check(lib().fv_bsr_spmv_t_mapped(nb, b, ptr(tp), ptr(ti), ptr(tb), ptr(vals), ptr(x),
                                     ptr(want), f64, st))
    tvals = torch.empty_like(vals)
    check(lib().fv_bsr_transpose_blocks(nnzb, b, ptr(tb), ptr(vals), ptr(tvals), f64, st))
    got = torch.empty_like(x)
    fn = lib().fv_bsr_spmv_f64 if f64 else lib().fv_bsr_spmv_f32
    check(fn(nb, b, ptr(tp), ptr(ti), ptr(tvals), ptr(x), ptr(got), 0, st))
    assert torch.equal(got, want)
    blocks = vals.view(nnzb, b, b)[tb.long()].transpose(1, 2).reshape(-1)
    assert torch.equal(tvals, blocks)


def test_dot_is_deterministic():
    from aquaflux_gb300.sparse import dot

    x = torch.randn(1_000_003, dtype=torch.float64, device="cuda")
    y = torch.randn(1_000_003, dtype=torch.float64, device="cuda")
    a, b = dot(x, y), dot(x, y)
    assert float(a) == float(b)
    assert abs(float(a) - float(torch.dot(x, y))) <= 1e-10 * float(torch.dot(x.abs(), y.abs()))


@pytest.mark.parametrize("precision", [32, 64])
def test_block_solve_pivot_quotients_are_correctly_rounded(precision):
    """The block backward sweep and the transposed forward sweep divide by their pivots through a
    corrected reciprocal; on a matrix of diagonal blocks both solves are x = r / d entry by entry
    and must equal IEEE division."""
    from aquaflux_gb300.ilu0 import Ilu0

    b, n = 6, 50000
    dt = np.float32 if precision == 32 else np.float64
    span = 12 if precision == 32 else 100
    rng = np.random.default_rng(7)

    def values(size):
        return (rng.choice([-1.0, 1.0], size) * 10.0 ** rng.uniform(-span, span, size)).astype(dt)

    d = values(n * b)
    r = values(n * b)
    # mantissas near the binade ends, where a quotient from a plain product is often off by one
    d[:1000] = (1.0 + rng.integers(0, 64, 1000) * np.finfo(dt).eps).astype(dt)
    r[:1000] = (2.0 - rng.integers(1, 64, 1000) * np.finfo(dt).eps).astype(dt)
    blocks = np.zeros((n, b, b))
    blocks[:, np.arange(b), np.arange(b)] = d.reshape(n, b)
    ip = np.arange(n + 1, dtype=np.int32)
    ix = np.arange(n, dtype=np.int32)
    f = Ilu0.from_csr(ip, ix, blocks.reshape(-1), block_size=b, precision=precision)
    got = f.solve(torch.tensor(r, device="cuda")).cpu().numpy()
    assert np.array_equal(got, r / d)
    got_t = f.solve(torch.tensor(r, device="cuda"), transpose=True).cpu().numpy()
    assert np.array_equal(got_t, r / d)


def test_block_ilu0_fp64_bitwise_equals_the_reference_kernel_on_a_channel_jacobian():
    """The GPU fp64 block ILU(0) of the equilibrated cell-major channel Jacobian against the
    reference's own compiled kernel (``aquaflux/solve/_ilu0.pyx``, built from its source) on the
    same scalar operator: factor and transposed solve bit for bit."""
    import torch

    from aquaflux_gb300 import workloads
    from aquaflux_gb300.ilu0 import Ilu0
    from aquaflux_gb300.solve import BlockJacobian, ShiftedCellMajorOperator
    from tests.ilu_helpers import reference_factor_solve, reference_kernel

    mod = reference_kernel()
    if mod is None:
        pytest.skip("the reference's compiled ILU(0) is not built on this machine")
    wl = workloads.channel3d(10)
    case = wl.device_case()
    state = torch.tensor(wl.initial_state(noise=0.02), device="cuda")
    jac = BlockJacobian(case)
    vals, _ = ShiftedCellMajorOperator(jac, equilibrate=True).assemble(jac.materialize(state))
    b = jac.b
    f = Ilu0.from_csr(jac.indptr, jac.indices, vals.cpu().numpy(), block_size=b, precision=64)
    sp_ip, sp_ix, sp_vals = to_scalar(jac.indptr, jac.indices, vals.cpu().numpy(), b)
    rhs = np.random.default_rng(0).standard_normal(len(sp_ip) - 1)
    _, data, _, xt = reference_factor_solve(mod, sp_ip, sp_ix, sp_vals, rhs)
    _, _, gfac = to_scalar(jac.indptr, jac.indices, f.factor_values().cpu().numpy(), b)
    np.testing.assert_array_equal(gfac, data)
    np.testing.assert_array_equal(f.solve(rhs, transpose=True).cpu().numpy(), xt)


@pytest.mark.parametrize("precision", [32, 64])
def test_cloned_ilu0_equals_a_fresh_factor_bitwise(precision):
    """fv_ilu0_clone: a factor on the same pattern without re-analysis -- from a factor or from a
    structure-only template, after the source's transposed structures exist or before -- gives
    bitwise the fresh factor's values, solves and transposed solves; a template refuses to factor
    or solve."""
    from aquaflux_gb300._lib import FvError
    from aquaflux_gb300.ilu0 import Ilu0

    d = golden("ilu0")
    ip, ix, vals = cell_major(d["ilu_indptr"], d["ilu_indices"], d["ilu_values"], 40, 3)
    bp, bi, bv = to_bsr(ip, ix, vals, 3)
    rhs = d["ilu_rhs"]
    fresh = Ilu0.from_csr(bp, bi, bv, block_size=3, precision=precision)
    template = fresh.clone(0)
    fresh.solve(rhs, transpose=True)  # the source now holds the transposed structures too
    for src in (fresh, template):
        c = src.clone(precision)
        c.refactor(bv)
        assert torch.equal(c.factor_values(), fresh.factor_values())
        assert torch.equal(c.solve(rhs), fresh.solve(rhs))
        assert torch.equal(c.solve(rhs, transpose=True), fresh.solve(rhs, transpose=True))
    with pytest.raises(FvError):
        template.refactor(bv)
    with pytest.raises(FvError):
        template.solve(rhs)


@pytest.mark.parametrize("precision", [64, 32])
def test_two_colour_block_ilu0_fused_sweep(precision):
    """A red-black numbered 2D grid: the second colour's rows are the last forward and the first
    backward level, solved by one fused sweep.  fp64: factor bitwise the oracle's, solve within
    1e-13, transposed solve bitwise; fp32 within its rounding; the fused solve is bitwise the one
    of the same factor cloned from a structure-only template (same kernels) and run to run."""
    import scipy.sparse as sp

    from aquaflux_gb300.ilu0 import Ilu0

    nx, ny, b = 12, 10, 3
    rng = np.random.default_rng(4)
    cells = [(i, j) for i in range(nx) for j in range(ny)]
    order = sorted(range(nx * ny), key=lambda c: ((cells[c][0] + cells[c][1]) % 2, c))
    new = np.empty(nx * ny, dtype=np.int64)
    new[order] = np.arange(nx * ny)
    rows, cols = [], []
    for c, (i, j) in enumerate(cells):
        for di, dj in ((0, 0), (1, 0), (-1, 0), (0, 1), (0, -1)):
            if 0 <= i + di < nx and 0 <= j + dj < ny:
                rows.append(new[c])
                cols.append(new[(i + di) * ny + (j + dj)])
    pat = sp.coo_matrix((np.ones(len(rows)), (rows, cols)), shape=(nx * ny,) * 2).tocsr()
    pat.sort_indices()
    nb = pat.nnz
    blocks = rng.standard_normal((nb, b, b)) * 0.3
    bi = pat.indices.astype(np.int32)
    bp = pat.indptr.astype(np.int32)
    for r in range(nx * ny):
        q = bp[r] + int(np.searchsorted(bi[bp[r]:bp[r + 1]], r))
        blocks[q] += np.eye(b) * 4.0
    a = sp.bsr_matrix((blocks, bi, bp), shape=(nx * ny * b,) * 2).tocsr()
    a.sort_indices()
    rhs = rng.standard_normal(nx * ny * b)
    _, data, x, xt = oracle_factor_solve(a.indptr, a.indices, a.data, rhs)
    f = Ilu0.from_csr(bp, bi, blocks.reshape(-1), block_size=b, precision=precision)
    got = f.solve(rhs).cpu().numpy()
    assert np.array_equal(got, f.solve(rhs).cpu().numpy())
    c = f.clone(0).clone(precision)
    c.refactor(blocks.reshape(-1))
    assert np.array_equal(got, c.solve(rhs).cpu().numpy())
    if precision == 64:
        sp_ip, sp_ix, sp_data = to_scalar(bp, bi, f.factor_values().cpu().numpy(), b)
        np.testing.assert_array_equal(sp_data, data)
        np.testing.assert_allclose(got, x, rtol=1e-13, atol=1e-15)
        np.testing.assert_array_equal(f.solve(rhs, transpose=True).cpu().numpy(), xt)
    else:
        np.testing.assert_allclose(got, x, rtol=2e-5, atol=1e-6)
