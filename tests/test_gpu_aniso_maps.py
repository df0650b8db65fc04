"""Per-cell anisotropy constants (Ku1, Ku2, Kc1..Kc3 maps; native/backends/fdm/src/demag_fp32.cu:275-292,
reductions_fp64.cu) on the GPU against the FP64 oracle: H_eff, the uniaxial and cubic
energies, and a short trajectory."""
import numpy as np
import pytest

from fullmag_gb300 import _abi
from helpers import problem, rel_l2
from test_gpu_parity import make_pair

pytestmark = pytest.mark.gpu


def _maps(n, seed):
    rng = np.random.default_rng(seed)
    return dict(ku1_field=rng.uniform(2e3, 8e3, n), kc1_field=rng.uniform(-6e4, -2e4, n),
                kc2_field=rng.uniform(0.0, 1e4, n))


@pytest.mark.parametrize("with_mask", [False, True])
def test_heff_and_energies_with_maps(gpu_lib, oracle, with_mask):
    nx, ny, nz = 20, 12, 3
    n = nx * ny * nz
    kw = problem(nx, ny, nz, seed=81, ku1=5e3, ku2=1e3, u_axis=(0.0, 0.6, 0.8), kc1=-4e4, **_maps(n, 3))
    mask = (np.random.default_rng(9).random(n) > 0.15).astype(np.uint8) if with_mask else None
    gpu, orc = make_pair(oracle, kw, mask=mask)
    m = kw["m0"] if mask is None else kw["m0"] * mask[:, None]
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), orc.fields(m)["h_eff"]) < 1e-5
    st, ost = gpu.stats(), orc.observe()
    assert abs(st["anisotropy_energy_joules"] - ost["e_uniaxial"]) <= 1e-5 * abs(ost["e_uniaxial"])
    assert abs(st["cubic_energy_joules"] - ost["e_cubic"]) <= 1e-5 * abs(ost["e_cubic"])
    assert abs(st["total_energy_joules"] - ost["e_total"]) <= 1e-5 * abs(ost["e_total"])


def test_trajectory_with_maps(gpu_lib, oracle):
    nx, ny, nz = 24, 12, 2
    n = nx * ny * nz
    kw = problem(nx, ny, nz, seed=82, alpha=0.1, ku1=5e3, u_axis=(1.0, 0.0, 0.0), ku1_field=_maps(n, 4)["ku1_field"])
    gpu, orc = make_pair(oracle, kw, integrator=_abi.INTEGRATOR_RK4)
    for _ in range(20):
        sg = gpu.step(5e-14)
        so = orc.step(5e-14)
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 2e-5
    assert abs(sg["anisotropy_energy_joules"] - so["e_uniaxial"]) <= 1e-4 * abs(so["e_uniaxial"])


def test_cubic_map_with_uniform_uniaxial(gpu_lib, oracle):
    nx, ny, nz = 16, 10, 2
    n = nx * ny * nz
    mp = _maps(n, 5)
    kw = problem(nx, ny, nz, seed=83, ku1=4e3, u_axis=(0.0, 0.0, 1.0), kc1=-3e4, kc3_field=mp["kc2_field"])
    gpu, orc = make_pair(oracle, kw)
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), orc.fields(kw["m0"])["h_eff"]) < 1e-5
    st, ost = gpu.stats(), orc.observe()
    assert abs(st["anisotropy_energy_joules"] - ost["e_uniaxial"]) <= 1e-5 * abs(ost["e_uniaxial"])
    assert abs(st["cubic_energy_joules"] - ost["e_cubic"]) <= 1e-5 * abs(ost["e_cubic"])
