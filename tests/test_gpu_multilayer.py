"""Stacked multilayer plans through the drop-in, against the FP64 oracle given the same
combined grid, mask, region ids and exchange table: the reference runner's single-grid
multilayer CUDA path (crates/fullmag-runner/src/multilayer_cuda.rs:729-990), which
creates one backend for the combined plan and reads each layer's cells back out."""
import numpy as np
import pytest

from fullmag_gb300 import FdmBackend, _abi
from fullmag_gb300.multilayer import Layer, layer_field, stacked_plan
from helpers import MU0, random_unit, rel_l2

pytestmark = pytest.mark.gpu

D = (2e-9, 2e-9, 3e-9)


def layers_case(gap_cells):
    a = Layer((24, 16, 2), (0.0, 0.0, 0.0), random_unit(24 * 16 * 2, 1))
    mask_b = np.ones(16 * 12, dtype=bool)
    mask_b[::7] = False
    b = Layer((16, 12, 1), (4 * D[0], 2 * D[1], (2 + gap_cells) * D[2]), random_unit(16 * 12, 2), mask_b)
    return [a, b]


@pytest.mark.parametrize("gap_cells,precision", [(1, _abi.PRECISION_SINGLE), (0, _abi.PRECISION_SINGLE),
                                                 (1, _abi.PRECISION_DOUBLE)])
def test_stacked_layers_vs_oracle(gpu_lib, oracle, gap_cells, precision):
    layers = layers_case(gap_cells)
    p = stacked_plan(layers, D, 1.3e-11)
    nx, ny, nz = p.grid
    kw = dict(nx=nx, ny=ny, nz=nz, dx=D[0], dy=D[1], dz=D[2], ms=8e5, a_ex=1.3e-11, alpha=0.3, gamma=2.211e5,
              m0=p.m0, h_ext=(10e-3 / MU0, 5e-3 / MU0, 0.0), region_mask=p.region_mask, exchange_lut=p.exchange_lut)
    sp = oracle.newell_spectra(nx, ny, nz, *D)
    gpu = FdmBackend(**kw, integrator=_abi.INTEGRATOR_RK4, spectra=sp, active_mask=p.active_mask, precision=precision)
    orc = oracle.Problem(**kw, integrator=oracle.RK4, active_mask=p.active_mask)
    tol_h = 1e-5 if precision == _abi.PRECISION_SINGLE else 1e-10
    tol_m = 2e-5 if precision == _abi.PRECISION_SINGLE else 1e-9
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), orc.fields()["h_eff"]) < tol_h
    for _ in range(30):
        sg = gpu.step(5e-14)
        so = orc.step(5e-14)
    m_g, m_o = gpu.copy_field(_abi.OBSERVABLE_M), orc.get_m()
    for li in range(2):  # per-layer read-back, as the runner's observers do
        assert np.abs(layer_field(p, layers, m_g, li) - layer_field(p, layers, m_o, li)).max() < tol_m
    assert abs(sg["total_energy_joules"] - so["e_total"]) <= 10 * tol_h * abs(so["e_total"])
    assert np.all(m_g[p.active_mask == 0] == 0.0)
