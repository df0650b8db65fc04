"""Stacked multilayer plans (fullmag_gb300/multilayer.py) on the CPU: the combined grid,
mask, region ids, initial state and exchange table that the reference runner builds in
crates/fullmag-runner/src/multilayer_cuda.rs:729-900."""
import numpy as np
import pytest

from fullmag_gb300.multilayer import Layer, layer_field, stacked_plan
from helpers import random_unit

D = (2e-9, 2e-9, 3e-9)


def two_layers(gap_cells=1):
    a = Layer((8, 6, 2), (0.0, 0.0, 0.0), random_unit(96, 1))
    mask_b = np.ones(4 * 3 * 1, dtype=bool)
    mask_b[0] = False
    b = Layer((4, 3, 1), (2 * D[0], 1 * D[1], (2 + gap_cells) * D[2]), random_unit(12, 2), mask_b)
    return [a, b]


def test_stacked_plan_geometry():
    layers = two_layers()
    p = stacked_plan(layers, D, 1.3e-11, inter_region_exchange=[(1, 2, 0.5e-11)])
    assert p.grid == (8, 6, 4) and p.offsets == [(0, 0, 0), (2, 1, 3)]
    assert p.active_mask.sum() == 96 + 11
    assert set(np.unique(p.region_mask)) == {0, 1, 2}
    assert np.all(p.region_mask[p.active_mask == 0] == 0)
    # layer views give back each layer's initial state (masked cells zero)
    assert np.array_equal(layer_field(p, layers, p.m0, 0), layers[0].m0)
    vb = layer_field(p, layers, p.m0, 1)
    assert np.array_equal(vb[1:], layers[1].m0[1:]) and np.all(vb[0] == 0)
    assert p.exchange_lut[1, 1] == p.exchange_lut[2, 2] == 1.3e-11
    assert p.exchange_lut[1, 2] == p.exchange_lut[2, 1] == 0.5e-11 and p.exchange_lut[0, 1] == 0.0


def test_stacked_plan_rejects_overlap_and_fractional_offsets():
    a = Layer((4, 4, 1), (0.0, 0.0, 0.0), random_unit(16, 1))
    b = Layer((4, 4, 1), (D[0], 0.0, 0.0), random_unit(16, 2))
    with pytest.raises(ValueError, match="overlapping"):
        stacked_plan([a, b], D, 1e-11)
    c = Layer((4, 4, 1), (0.5 * D[0], 0.0, D[2]), random_unit(16, 3))
    with pytest.raises(ValueError, match="whole number"):
        stacked_plan([a, c], D, 1e-11)
