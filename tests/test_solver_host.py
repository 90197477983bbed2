"""Host-side pieces of the forward march that need no GPU."""
import pytest
import torch

from aquaflux_gb300.solve import positive_projection


def test_positive_projection_clips_only_decreasing_entries():
    """``positive_block_projection`` (aquaflux/solve/implicit.py:197-300): each entry of the block
    keeps at least (1 - tau) of its value (plus the floor's room); entries outside the block and
    increasing entries are untouched; a zero correction stays zero."""
    phi = torch.tensor([1.0, 2.0, 1e-3, 0.5, 7.0], dtype=torch.float64)
    delta = torch.tensor([-5.0, -1.0, -1.0, 0.3, -9.0], dtype=torch.float64)
    out = positive_projection(phi, delta, 1, 4, tau=0.9)
    assert out[0] == -5.0 and out[4] == -9.0  # outside the block
    assert out[1] == -1.0  # within reach
    assert torch.isclose(out[2], torch.tensor(-0.9e-3, dtype=torch.float64))
    assert out[3] == 0.3
    assert bool((phi[1:4] + out[1:4] > 0).all())
    floored = positive_projection(phi, delta, 1, 4, tau=0.9, floor=1.0)
    assert torch.isclose(floored[2], torch.tensor(-0.9 * (1e-3 + 1.0), dtype=torch.float64))
    zero = positive_projection(phi, torch.zeros(5, dtype=torch.float64), 0, 5)
    assert bool((zero == 0).all())


def test_reynolds_scales_are_geometric_and_end_at_the_target():
    """GeometricReynoldsSchedule.scales (aquaflux/turbulence/reynolds.py:96-132)."""
    from aquaflux_gb300.solve import reynolds_scales

    assert reynolds_scales(0) == (1.0,)
    assert reynolds_scales(1) == (10.0, 1.0)
    assert reynolds_scales(2) == (100.0, 10.0, 1.0)
    assert reynolds_scales(2, ratio=3.0) == (9.0, 3.0, 1.0)
    with pytest.raises(ValueError):
        reynolds_scales(-1)
