"""The allocation-free transposed BSR SpMV against the allocating one, through the C ABI.

``fv_bsr_spmv_t_f64_noalloc`` exists for callers that cannot allocate device memory while they
run (an FFI call inside a framework that owns the device memory, an embedded solver that forbids
allocation after start-up).  Its transpose map lives in one fixed static device array shared by
every call, so this test makes two calls in a row with different operators to show the array is
re-initialised, and compares each with ``fv_bsr_spmv_f64(transpose=1)``.  Both sum each column's
products in ascending row order with the same rounding (both units built with ``-fmad=false``),
so the comparison is bitwise.  It is collected last so that a run stopping at the first
failure has already run every other test; it passes alone in a fresh process too.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _pattern(nb, density, seed):
    import scipy.sparse as sp

    a = sp.random(nb, nb, density=density, random_state=seed, format="csr") + sp.eye(nb)
    a = a.tocsr()
    a.sort_indices()
    return a.indptr.astype(np.int32), a.indices.astype(np.int32)


def _call(fn_name, *args):
    from aquaflux_gb300 import _lib

    L = _lib.lib()
    _lib.check(getattr(L, fn_name)(*args))


def test_no_alloc_transpose_spmv_matches_allocating_path_twice():
    from aquaflux_gb300._lib import ptr

    stream = torch.cuda.current_stream().cuda_stream
    for call, (nb, b, density) in enumerate([(700, 3, 0.01), (450, 6, 0.02)]):
        ip, ix = _pattern(nb, density, seed=call)
        rng = np.random.default_rng(call)
        nnzb = int(ip[-1])
        vals = torch.tensor(rng.standard_normal(nnzb * b * b), device="cuda")
        x = torch.tensor(rng.standard_normal(nb * b), device="cuda")
        d_ip = torch.tensor(ip, device="cuda")
        d_ix = torch.tensor(ix, device="cuda")
        y_ref = torch.empty(nb * b, dtype=torch.float64, device="cuda")
        y_new = torch.full((nb * b,), float("nan"), dtype=torch.float64, device="cuda")
        _call("fv_bsr_spmv_f64", nb, b, ptr(d_ip), ptr(d_ix), ptr(vals), ptr(x), ptr(y_ref), 1,
              stream)
        _call("fv_bsr_spmv_t_f64_noalloc", nb, nnzb, b, ptr(d_ip), ptr(d_ix), ptr(vals), ptr(x),
              ptr(y_new), stream)
        torch.cuda.synchronize()
        ref, new = y_ref.cpu().numpy(), y_new.cpu().numpy()
        assert np.isfinite(new).all()
        np.testing.assert_array_equal(new, ref)


def test_no_alloc_marks_an_inconsistent_nnzb_with_nan():
    """nnzb must equal indptr[n]: a smaller or larger value gives an all-NaN y, not a silently
    truncated product; the next consistent call is exact again."""
    from aquaflux_gb300._lib import ptr

    stream = torch.cuda.current_stream().cuda_stream
    nb, b = 300, 3
    ip, ix = _pattern(nb, 0.02, seed=5)
    rng = np.random.default_rng(5)
    nnzb = int(ip[-1])
    vals = torch.tensor(rng.standard_normal(nnzb * b * b), device="cuda")
    x = torch.tensor(rng.standard_normal(nb * b), device="cuda")
    d_ip = torch.tensor(ip, device="cuda")
    d_ix = torch.tensor(ix, device="cuda")
    y = torch.zeros(nb * b, dtype=torch.float64, device="cuda")
    for wrong in (nnzb - 7, nnzb + 7):
        _call("fv_bsr_spmv_t_f64_noalloc", nb, wrong, b, ptr(d_ip), ptr(d_ix), ptr(vals), ptr(x),
              ptr(y), stream)
        torch.cuda.synchronize()
        assert torch.isnan(y).all()
    y_ref = torch.empty_like(y)
    _call("fv_bsr_spmv_f64", nb, b, ptr(d_ip), ptr(d_ix), ptr(vals), ptr(x), ptr(y_ref), 1, stream)
    _call("fv_bsr_spmv_t_f64_noalloc", nb, nnzb, b, ptr(d_ip), ptr(d_ix), ptr(vals), ptr(x),
          ptr(y), stream)
    torch.cuda.synchronize()
    assert torch.equal(y, y_ref)


def test_no_alloc_rejects_patterns_beyond_its_scratch():
    from aquaflux_gb300 import _lib
    from aquaflux_gb300._lib import ptr

    nb, b = 4, 1
    d_ip = torch.tensor([0, 1, 2, 3, 4], dtype=torch.int32, device="cuda")
    d_ix = torch.tensor([0, 1, 2, 3], dtype=torch.int32, device="cuda")
    vals = torch.ones(4, dtype=torch.float64, device="cuda")
    x = torch.ones(4, dtype=torch.float64, device="cuda")
    y = torch.empty(4, dtype=torch.float64, device="cuda")
    L = _lib.lib()
    rc = L.fv_bsr_spmv_t_f64_noalloc(nb, 3_000_000, b, ptr(d_ip), ptr(d_ix), ptr(vals), ptr(x),
                                     ptr(y), torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.FV_ERR_ARG
    assert b"scratch" in L.fv_last_error()
