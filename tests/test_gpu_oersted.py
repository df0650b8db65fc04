"""Oersted field of a cylindrical conductor on the GPU against the FP64 oracle
(native/backends/fdm/src/context.cu:844-905, demag_fp32.cu:585-616): the field in H_eff
(not in any energy), constant, sinusoidal and pulsed currents along trajectories of each
integrator, with the reference's rule for the time at which each evaluation sees the current."""
import numpy as np
import pytest

from fullmag_gb300 import FdmBackend, FdmError, _abi
from helpers import problem, rel_l2
from test_gpu_parity import make_pair

pytestmark = pytest.mark.gpu

OE = dict(oersted_current=5e-3, oersted_radius=20e-9, oersted_center=(48e-9, 24e-9, 0.0))


def test_heff_and_energy(gpu_lib, oracle):
    kw = problem(24, 12, 2, seed=91, **OE)
    mask = (np.random.default_rng(2).random(24 * 12 * 2) > 0.1).astype(np.uint8)
    gpu, orc = make_pair(oracle, kw, mask=mask)
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), orc.fields(kw["m0"] * mask[:, None])["h_eff"]) < 1e-5
    st, ost = gpu.stats(), orc.observe()
    assert abs(st["external_energy_joules"] - ost["e_external"]) <= 1e-5 * abs(ost["e_external"])


@pytest.mark.parametrize("integrator,kind", [(_abi.INTEGRATOR_RK4, 1), (_abi.INTEGRATOR_HEUN, 2),
                                             (_abi.INTEGRATOR_ABM3, 1)])
def test_time_dependent_trajectory(gpu_lib, oracle, integrator, kind):
    extra = dict(oersted_kind=kind, oersted_freq=2e11, oersted_phase=0.3, oersted_offset=0.1,
                 oersted_t_on=2e-13, oersted_t_off=6e-13)
    kw = problem(24, 12, 2, seed=92, alpha=0.1, **OE, **extra)
    kw["oersted_current"] = 5e-2
    gpu, orc = make_pair(oracle, kw, integrator=integrator)
    for _ in range(20):
        sg = gpu.step(5e-14)
        so = orc.step(5e-14)
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 2e-5
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), orc.fields(orc.get_m())["h_eff"]) < 1e-5


def test_dp45_sinusoidal(gpu_lib, oracle):
    kw = problem(32, 16, 1, seed=93, alpha=0.1, adaptive_max_error=1e-5, oersted_kind=1, oersted_freq=2e11,
                 **OE)
    kw["oersted_current"] = 5e-2
    gpu, orc = make_pair(oracle, kw, integrator=_abi.INTEGRATOR_DP45)
    dt_g = dt_o = 1e-13
    for _ in range(10):
        sg = gpu.step(dt_g)
        so = orc.step(dt_o)
        dt_g, dt_o = sg["suggested_next_dt"], so["suggested_next_dt"]
    assert abs(sg["time_seconds"] - so["time"]) <= 1e-3 * so["time"]
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 1e-3


def test_nonpositive_radius_is_rejected(gpu_lib):
    with pytest.raises(FdmError):
        FdmBackend(**problem(8, 4, 1, seed=94, oersted_current=1e-3, oersted_radius=0.0))
