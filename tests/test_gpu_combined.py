"""Every term of the extra-field pass at once, with a mask, on the GPU against the FP64
oracle: interfacial DMI, magnetoelastic field, exchange with region ids and a table,
per-cell uniaxial anisotropy, spin-orbit torque, a sinusoidal Oersted current and the
thermal field.  Each term is checked on its own in its own file; this checks that they
share the pass (one output, one set of FP64 sums) without interfering."""
import numpy as np
import pytest

from fullmag_gb300 import _abi
from helpers import problem, rel_l2
from test_gpu_parity import make_pair

pytestmark = pytest.mark.gpu


def _all_terms(nx, ny, nz, seed):
    n = nx * ny * nz
    rng = np.random.default_rng(seed)
    x = np.tile(np.arange(nx), ny * nz)
    reg = np.where(x < nx // 2, 1, 2).astype(np.uint32)
    lut = np.zeros((256, 256))
    lut[1, 1], lut[2, 2], lut[1, 2], lut[2, 1] = 1.3e-11, 0.9e-11, 0.4e-11, 0.4e-11
    return dict(dmi_d_interfacial=1.5e-3, mel_b1=-3e6, mel_b2=2e6, mel_strain=(1e-3, -5e-4, 2e-4, 1e-4, 0.0, 3e-4),
                region_mask=reg, exchange_lut=lut, ku1=4e3, u_axis=(0.0, 0.0, 1.0),
                ku1_field=rng.uniform(2e3, 6e3, n), sot_je=1e16, sot_xi_dl=0.2, sot_xi_fl=0.05,
                sot_sigma=(0.0, 1.0, 0.0), sot_thickness=2e-9, oersted_current=2e-2, oersted_radius=15e-9,
                oersted_center=(40e-9, 20e-9, 0.0), oersted_kind=1, oersted_freq=1e11, temperature=20.0)


def test_fields_and_energies(gpu_lib, oracle):
    nx, ny, nz = 20, 12, 2
    kw = problem(nx, ny, nz, seed=121, alpha=0.1, **_all_terms(nx, ny, nz, 5))
    mask = (np.random.default_rng(10).random(nx * ny * nz) > 0.1).astype(np.uint8)
    gpu, orc = make_pair(oracle, kw, mask=mask)
    ref = orc.fields(kw["m0"] * mask[:, None])
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), ref["h_eff"]) < 1e-5
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EX), ref["h_ex"]) < 1e-5
    st, ost = gpu.stats(), orc.observe()
    for a, b in (("exchange_energy_joules", "e_exchange"), ("dmi_energy_joules", "e_dmi"),
                 ("anisotropy_energy_joules", "e_uniaxial"), ("external_energy_joules", "e_external"),
                 ("total_energy_joules", "e_total")):
        assert abs(st[a] - ost[b]) <= 1e-5 * abs(ost[b]) + 1e-30, a


@pytest.mark.parametrize("integrator", [_abi.INTEGRATOR_RK4, _abi.INTEGRATOR_HEUN])
def test_trajectory(gpu_lib, oracle, integrator):
    nx, ny, nz = 20, 12, 2
    kw = problem(nx, ny, nz, seed=122, alpha=0.1, **_all_terms(nx, ny, nz, 6))
    mask = (np.random.default_rng(11).random(nx * ny * nz) > 0.1).astype(np.uint8)
    gpu, orc = make_pair(oracle, kw, integrator=integrator, mask=mask)
    for _ in range(15):
        sg = gpu.step(4e-14)
        so = orc.step(4e-14)
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 3e-5
    assert abs(sg["max_rhs_amplitude"] - so["max_rhs"]) <= 1e-4 * so["max_rhs"]
    assert abs(sg["total_energy_joules"] - so["e_total"]) <= 1e-4 * abs(so["e_total"])


@pytest.mark.parametrize("shape", [(7, 5, 3), (9, 1, 1), (1, 1, 1), (1, 7, 1), (5, 1, 4), (3, 4, 2)])
def test_edge_shapes(gpu_lib, oracle, shape):
    # extents of 1 clamp every neighbour of DMI and region exchange to the cell itself
    nx, ny, nz = shape
    n = nx * ny * nz
    terms = _all_terms(nx, ny, nz, 7)
    terms["region_mask"] = (np.arange(n) % 3).astype(np.uint32)
    lut = terms["exchange_lut"]
    lut[0, 0], lut[0, 1], lut[1, 0], lut[0, 2], lut[2, 0] = 1.1e-11, 0.2e-11, 0.2e-11, 0.6e-11, 0.6e-11
    kw = problem(nx, ny, nz, seed=123, alpha=0.1, d=(3e-9, 2e-9, 2.5e-9), **terms)
    mask = np.ones(n, dtype=np.uint8)
    if n > 2:
        mask[n // 2] = 0
    gpu, orc = make_pair(oracle, kw, mask=mask)
    ref = orc.fields(kw["m0"] * mask[:, None])
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), ref["h_eff"]) < 1e-5
    h_ex = gpu.copy_field(_abi.OBSERVABLE_H_EX)
    assert np.abs(h_ex - ref["h_ex"]).max() <= 1e-5 * max(np.abs(ref["h_ex"]).max(), 1.0)
    for _ in range(5):
        sg = gpu.step(4e-14)
        so = orc.step(4e-14)
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 2e-5
    assert abs(sg["total_energy_joules"] - so["e_total"]) <= 1e-4 * abs(so["e_total"]) + 1e-30
