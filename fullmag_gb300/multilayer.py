"""Stacked multilayer problems on one grid, the way the reference runner drives several
bodies through the single-grid C ABI (crates/fullmag-runner/src/multilayer_cuda.rs:729-900,
build_native_stacked_cuda_plan, then NativeFdmBackend::create at :907).

All layers share the material and the cell size.  The global grid is the bounding box
of the layers (origins and extents must fall on whole cells); each layer's active cells
are placed at its offset, the active mask is their union (an overlap is an error), the
region id of a cell is its layer index + 1 (0 outside every layer), and the exchange
table couples a region only with itself (A on the diagonal, native_fdm.rs:216-236), so
layers interact through the demag field alone unless the caller adds inter-region
stiffness.  The plan goes through the same C ABI as a single body; per-layer outputs are
views of the global fields."""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

MAX_REGIONS = 256


@dataclass
class Layer:
    grid: Tuple[int, int, int]                 # cells (nx, ny, nz)
    origin: Tuple[float, float, float]         # metres
    m0: np.ndarray                             # (nx*ny*nz, 3)
    mask: Optional[np.ndarray] = None          # optional per-cell bool (layer-local order)


@dataclass
class StackedPlan:
    grid: Tuple[int, int, int]
    offsets: List[Tuple[int, int, int]]
    active_mask: np.ndarray                    # uint8, global
    region_mask: np.ndarray                    # uint32, global
    m0: np.ndarray                             # (n, 3), global
    exchange_lut: np.ndarray                   # 256 x 256

    def layer_indices(self, layer: Layer, offset: Tuple[int, int, int]) -> np.ndarray:
        """Global cell indices of a layer's cells, in the layer's x-fastest order."""
        nx, ny, nz = layer.grid
        gx, gy, _ = self.grid
        z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        return (((z + offset[2]) * gy + (y + offset[1])) * gx + (x + offset[0])).reshape(-1)


def _cells(v: float, d: float, what: str) -> int:
    c = v / d
    r = round(c)
    if abs(c - r) > 1e-6 or r < 0:
        raise ValueError(f"{what} is not a whole number of cells")
    return int(r)


def stacked_plan(layers: Sequence[Layer], cell: Tuple[float, float, float], a_ex: float,
                 inter_region_exchange: Sequence[Tuple[int, int, float]] = ()) -> StackedPlan:
    if not layers:
        raise ValueError("no layers")
    lo = [min(l.origin[a] for l in layers) for a in range(3)]
    hi = [max(l.origin[a] + l.grid[a] * cell[a] for l in layers) for a in range(3)]
    grid = tuple(_cells(hi[a] - lo[a], cell[a], "global extent") for a in range(3))
    if min(grid) < 1:
        raise ValueError("empty global grid")
    gx, gy, gz = grid
    n = gx * gy * gz
    active = np.zeros(n, dtype=np.uint8)
    region = np.zeros(n, dtype=np.uint32)
    m0 = np.zeros((n, 3))
    plan = StackedPlan(grid, [], active, region, m0, np.zeros((MAX_REGIONS, MAX_REGIONS)))
    for li, layer in enumerate(layers):
        off = tuple(_cells(layer.origin[a] - lo[a], cell[a], "layer offset") for a in range(3))
        if any(off[a] + layer.grid[a] > grid[a] for a in range(3)):
            raise ValueError("layer outside the global grid")
        plan.offsets.append(off)
        idx = plan.layer_indices(layer, off)
        on = np.ones(idx.size, dtype=bool) if layer.mask is None else np.asarray(layer.mask, dtype=bool).reshape(-1)
        g = idx[on]
        if np.any(active[g]):
            raise ValueError(f"overlapping active cells between bodies (layer {li})")
        active[g] = 1
        region[g] = li + 1
        m0[g] = np.asarray(layer.m0, dtype=np.float64).reshape(-1, 3)[on]
    for r in range(MAX_REGIONS):
        plan.exchange_lut[r, r] = a_ex
    for ri, rj, a in inter_region_exchange:
        plan.exchange_lut[ri, rj] = plan.exchange_lut[rj, ri] = a
    return plan


def layer_field(plan: StackedPlan, layers: Sequence[Layer], field: np.ndarray, li: int) -> np.ndarray:
    """A layer's part of a global (n, 3) field, in the layer's cell order."""
    return np.asarray(field).reshape(-1, 3)[plan.layer_indices(layers[li], plan.offsets[li])]
