"""The staleness triggers as pure functions of a step history (``aquaflux/solve/march.py:
130-285``): the same histories give the reference's answers."""
from aquaflux_gb300.refresh import CoefficientDriftTrigger, CycleGrowthTrigger, StepReport


def _hist(cycles, ratios=None, drift=None):
    ratios = ratios or [1e-3] * len(cycles)
    drift = drift or [0.0] * len(cycles)
    return [StepReport(i, c, r, r, d) for i, (c, r, d) in enumerate(zip(cycles, ratios, drift))]


def test_cycle_growth_needs_warmup_gate_and_patience():
    t = CycleGrowthTrigger()  # growth 2, gate 5e-2, warmup 5, patience 2
    assert not t.should_refresh(_hist([10, 10, 10, 10, 20]))          # within the warmup
    assert t.should_refresh(_hist([10, 10, 10, 10, 10, 20, 20]))
    assert not t.should_refresh(_hist([10, 10, 10, 10, 10, 10, 20]))  # one step: no patience
    assert not t.should_refresh(_hist([10, 10, 10, 10, 10, 20, 19]))  # below 2x the minimum
    # the developed-flow gate: the latest residual ratio must be at most 5e-2
    assert not t.should_refresh(_hist([10] * 5 + [20, 20], ratios=[1e-3] * 6 + [0.1]))


def test_cycle_growth_baseline_skips_zero_counts():
    t = CycleGrowthTrigger()
    # zeros are "no measurement": they neither set the minimum nor count as grown
    assert t.should_refresh(_hist([0, 10, 0, 10, 10, 20, 20]))
    assert not t.should_refresh(_hist([10, 10, 10, 10, 10, 20, 0]))
    assert not t.should_refresh(_hist([0] * 8))


def test_coefficient_drift_fires_at_the_threshold_after_warmup():
    t = CoefficientDriftTrigger()  # threshold 0.1, warmup 3
    assert not t.should_refresh(_hist([5] * 3, drift=[0.0, 0.2, 0.3]))
    assert t.should_refresh(_hist([5] * 4, drift=[0.0, 0.0, 0.0, 0.1]))
    assert not t.should_refresh(_hist([5] * 4, drift=[0.5, 0.5, 0.5, 0.09]))
