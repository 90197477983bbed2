"""Evaluation-order choices change which thread evaluates a cell or face, never the arithmetic: the
warp-coherent cell order and the per-stage block sizes of the autotuner give residual, JVP (fp64
and fp32 tangents), VJP and the node adjoint bitwise equal to the natural order at one block
size."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from cases import device_case

pytestmark = pytest.mark.gpu


def _evaluations(fc, s, v, w):
    out = {"residual": fc.residual(s).cpu().numpy(),
           "jvp": fc.jvp(s, v).cpu().numpy(),
           "jvp32": fc.jvp(s, v, precision=32).cpu().numpy(),
           "vjp": fc.vjp(s, w).cpu().numpy()}
    return out


def _both_orders(fc, s, v, w):
    n = fc.set_cell_order(False)
    natural = _evaluations(fc, s, v, w)
    assert fc.set_cell_order(True) == n
    coherent = _evaluations(fc, s, v, w)
    return n, natural, coherent


def test_renumbered_sst_channel_is_bitwise_order_independent():
    from aquaflux_gb300 import workloads

    wl = workloads.channel3d(10, renumber="host")
    fc = wl.device_case()
    rng = np.random.default_rng(5)
    s = wl.initial_state() * (1.0 + 0.05 * rng.standard_normal(fc.n_unknowns))
    v = rng.standard_normal(fc.n_unknowns)
    w = rng.standard_normal(fc.n_unknowns)
    n, natural, coherent = _both_orders(fc, s, v, w)
    # interior, and per boundary pattern (faces, corners) of the six patches
    assert n > 6
    for k in natural:
        assert np.array_equal(natural[k], coherent[k]), k


@pytest.mark.parametrize("name", ["ccavj", "lcavj", "csst3", "psst2"])
def test_reference_cases_are_bitwise_order_independent(name):
    fc, case, d, p = device_case(name)
    s = d[p + "states"][0]
    rng = np.random.default_rng(7)
    v = rng.standard_normal(s.size)
    w = rng.standard_normal(s.size)
    _, natural, coherent = _both_orders(fc, s, v, w)
    for k in natural:
        assert np.array_equal(natural[k], coherent[k]), (name, k)


def test_node_adjoint_is_bitwise_order_independent():
    fc, case, d, p = device_case("csst3")
    s = d[p + "states"][0]
    w = np.random.default_rng(9).standard_normal(s.size)
    fc.set_cell_order(False)
    a = fc.node_vjp(s, w).cpu().numpy()
    fc.set_cell_order(True)
    b = fc.node_vjp(s, w).cpu().numpy()
    assert np.array_equal(a, b)


def test_per_stage_block_sizes_are_bitwise_neutral():
    from aquaflux_gb300 import workloads

    wl = workloads.channel3d(10, renumber="host")
    fc = wl.device_case()
    rng = np.random.default_rng(11)
    s = wl.initial_state() * (1.0 + 0.05 * rng.standard_normal(fc.n_unknowns))
    v = rng.standard_normal(fc.n_unknowns)
    w = rng.standard_normal(fc.n_unknowns)
    fc.set_block_size(128)
    assert fc.block_sizes() == [128] * len(fc.STAGES)
    ref = _evaluations(fc, s, v, w)
    best = fc.autotune(s, w)
    sizes = fc.block_sizes()
    assert best in (32, 64, 96, 128) and all(t in (32, 64, 96, 128) for t in sizes)
    got = _evaluations(fc, s, v, w)
    for k in ref:
        assert np.array_equal(ref[k], got[k]), k
