"""DMI (interfacial, bulk) and magnetoelastic terms on the GPU against the FP64 oracle
(native/backends/fdm/src/demag_fp32.cu:319-376, reductions_fp64.cu:647-720): H_eff per
evaluation, the DMI and Zeeman energies (also with a field map), short trajectories, and
the batch driver's per-problem path."""
import numpy as np
import pytest

from fullmag_gb300 import FdmBackend, FdmBatch, FdmError, _abi
from helpers import MU0, problem, rel_l2
from test_gpu_parity import make_pair

pytestmark = pytest.mark.gpu

STRAIN = (1e-3, -2e-4, 3e-4, 4e-4, -6e-4, 8e-4)


def _kw(nx, ny, nz, seed, **extra):
    args = dict(alpha=0.2, dmi_d_interfacial=3e-3, dmi_d_bulk=1.5e-3, mel_b1=5e6, mel_b2=7e6, mel_strain=STRAIN)
    args.update(extra)
    return problem(nx, ny, nz, seed=seed, **args)


@pytest.mark.parametrize("with_mask", [False, True])
def test_heff_and_energies(gpu_lib, oracle, with_mask):
    kw = _kw(20, 12, 3, seed=61)
    mask = None
    if with_mask:
        mask = (np.random.default_rng(3).random(20 * 12 * 3) > 0.12).astype(np.uint8)
    gpu, orc = make_pair(oracle, kw, mask=mask)
    m = kw["m0"] if mask is None else kw["m0"] * mask[:, None]
    ref = orc.fields(m)
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), ref["h_eff"]) < 1e-5
    st, ost = gpu.stats(), orc.observe()
    assert abs(st["dmi_energy_joules"] - ost["e_dmi"]) <= 1e-5 * abs(ost["e_dmi"])
    assert abs(st["external_energy_joules"] - ost["e_external"]) <= 1e-5 * abs(ost["e_external"])
    assert abs(st["total_energy_joules"] - ost["e_total"]) <= 1e-5 * abs(ost["e_total"])


def test_field_map_with_dmi_keeps_zeeman_energy(gpu_lib, oracle):
    kw = _kw(16, 10, 2, seed=62, b_mt=None)
    gpu, orc = make_pair(oracle, kw)
    hmap = np.random.default_rng(5).normal(0.0, 3e-3, size=(16 * 10 * 2, 3)) / MU0
    gpu.set_field_map(hmap)
    orc.set_field_map(hmap)
    gpu.refresh()
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), orc.fields(kw["m0"])["h_eff"]) < 1e-5
    st, ost = gpu.stats(), orc.observe()
    assert abs(st["external_energy_joules"] - ost["e_external"]) <= 1e-5 * abs(ost["e_external"])
    assert abs(st["dmi_energy_joules"] - ost["e_dmi"]) <= 1e-5 * abs(ost["e_dmi"])


def test_rk4_trajectory(gpu_lib, oracle):
    kw = _kw(24, 12, 2, seed=63)
    gpu, orc = make_pair(oracle, kw, integrator=_abi.INTEGRATOR_RK4)
    for _ in range(20):
        sg = gpu.step(5e-14)
        so = orc.step(5e-14)
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 2e-5
    assert abs(sg["dmi_energy_joules"] - so["e_dmi"]) <= 1e-4 * abs(so["e_dmi"])
    assert abs(sg["total_energy_joules"] - so["e_total"]) <= 1e-4 * abs(so["e_total"])


def test_thin_film_interfacial_dp45(gpu_lib, oracle):
    kw = problem(32, 16, 1, seed=64, alpha=0.1, dmi_d_interfacial=3e-3, adaptive_max_error=1e-5)
    gpu, orc = make_pair(oracle, kw, integrator=_abi.INTEGRATOR_DP45)
    dt_g = dt_o = 1e-13
    for _ in range(10):
        sg = gpu.step(dt_g)
        so = orc.step(dt_o)
        dt_g, dt_o = sg["suggested_next_dt"], so["suggested_next_dt"]
    assert abs(sg["time_seconds"] - so["time"]) <= 1e-3 * so["time"]
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 1e-3


def test_batch_and_adjoint_with_dmi(gpu_lib):
    ps = []
    for i, (nx, ny, nz) in enumerate([(17, 9, 1), (12, 10, 2)]):
        kw = problem(nx, ny, nz, seed=65 + i, alpha=0.1, dmi_d_interfacial=2e-3)
        kw["integrator"] = _abi.INTEGRATOR_DP45
        kw["adaptive_max_error"] = 1e-5
        ps.append(kw)
    batch = FdmBatch(ps)
    steps, _ = batch.step_until(1e-12, 1e-13)
    for i, kw in enumerate(ps):
        be = FdmBackend(**kw)
        t, dt, n = 0.0, 1e-13, 0
        while t < 1e-12 * (1 - 1e-12):
            st = be.step(min(dt, 1e-12 - t))
            t, dt, n = st["time_seconds"], st["suggested_next_dt"], n + 1
        assert steps[i] == n
        assert np.abs(batch.copy_field(i) - be.copy_field(_abi.OBSERVABLE_M)).max() < 1e-6
        be.close()
    batch.close()
    kw = dict(ps[0])
    kw["integrator"] = _abi.INTEGRATOR_RK4
    be = FdmBackend(**kw)
    with pytest.raises(FdmError):
        be.adjoint_forward(5e-14, 4)
