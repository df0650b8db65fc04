"""RK23 and ABM3 on the GPU against the FP64 oracle (native/backends/fdm/src/llg_rk23_fp32.cu,
native/backends/fdm/src/llg_abm3_fp32.cu): adaptive Bogacki-Shampine trajectories with
the ABI's step control, ABM3 with its Heun start-up, its restart after a step size
change and after an upload, and both through the batch driver."""
import numpy as np
import pytest

from fullmag_gb300 import FdmBackend, FdmBatch, _abi
from helpers import problem
from test_gpu_parity import make_pair

pytestmark = pytest.mark.gpu


def test_rk23_trajectory(gpu_lib, oracle):
    kw = problem(24, 12, 2, seed=51, alpha=0.05, ku1=5e3, u_axis=(1, 0, 0), b_mt=(-20.0, 5.0, 0.0),
                 adaptive_max_error=1e-5)
    gpu, orc = make_pair(oracle, kw, integrator=_abi.INTEGRATOR_RK23)
    dt_g = dt_o = 1e-13
    rej = 0
    for _ in range(25):
        sg = gpu.step(dt_g)
        so = orc.step(dt_o)
        rej += so["rejected_attempts"]
        dt_g, dt_o = sg["suggested_next_dt"], so["suggested_next_dt"]
    assert sg["step"] == 25
    assert abs(sg["time_seconds"] - so["time"]) <= 1e-3 * so["time"]
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 1e-3
    assert abs(sg["total_energy_joules"] - so["e_total"]) <= 1e-3 * abs(so["e_total"])
    assert 0.2 * dt_o < dt_g < 5.0 * dt_o


def test_rk23_first_step_matches_oracle_closely(gpu_lib, oracle):
    """One accepted step from the same state: same step size, state within FP32 error."""
    kw = problem(16, 8, 2, seed=52, adaptive_max_error=1e-4)
    gpu, orc = make_pair(oracle, kw, integrator=_abi.INTEGRATOR_RK23)
    sg, so = gpu.step(2e-14), orc.step(2e-14)
    assert sg["dt_seconds"] == so["dt_used"]
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 2e-6
    assert abs(sg["suggested_next_dt"] - so["suggested_next_dt"]) <= 1e-3 * so["suggested_next_dt"]


def test_abm3_trajectory_startup_and_restart(gpu_lib, oracle):
    kw = problem(32, 16, 2, seed=53, alpha=0.3)
    gpu, orc = make_pair(oracle, kw, integrator=_abi.INTEGRATOR_ABM3)
    dt = 5e-14
    plan = [dt] * 12 + [1.5 * dt] * 6 + [1.55 * dt] * 4  # restart at 1.5 dt, none at +3 %
    for d in plan:
        sg = gpu.step(d)
        so = orc.step(d)
        assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 2e-5
    assert sg["step"] == len(plan)
    assert abs(sg["time_seconds"] - sum(plan)) < 1e-24
    assert abs(sg["total_energy_joules"] - so["e_total"]) <= 1e-4 * abs(so["e_total"])
    assert abs(sg["max_rhs_amplitude"] - so["max_rhs"]) <= 1e-4 * so["max_rhs"]


def test_abm3_restarts_after_upload(gpu_lib, oracle):
    kw = problem(16, 8, 2, seed=54, alpha=0.3)
    gpu, orc = make_pair(oracle, kw, integrator=_abi.INTEGRATOR_ABM3)
    for _ in range(5):
        gpu.step(5e-14)
        orc.step(5e-14)
    m1 = problem(16, 8, 2, seed=55)["m0"]
    gpu.upload(m1)
    orc.set_m(m1)
    for _ in range(5):
        gpu.step(5e-14)
        orc.step(5e-14)
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 2e-5


def test_batch_runs_rk23_and_abm3(gpu_lib):
    """The batch driver steps RK23 (adaptive) and ABM3 (fixed) problems one attempt at a
    time; each must follow its single-problem trajectory."""
    for integrator, adaptive in ((_abi.INTEGRATOR_RK23, True), (_abi.INTEGRATOR_ABM3, False)):
        ps = []
        for i, (nx, ny, nz) in enumerate([(17, 9, 1), (12, 10, 2)]):
            kw = problem(nx, ny, nz, seed=56 + i, alpha=0.1)
            kw["integrator"] = integrator
            kw["adaptive_max_error"] = 1e-5
            ps.append(kw)
        batch = FdmBatch(ps)
        t_end, dt0 = 1e-12, 5e-14
        steps, _ = batch.step_until(t_end, dt0)
        for i, kw in enumerate(ps):
            be = FdmBackend(**kw)
            t, dt, n = 0.0, dt0, 0
            while t < t_end * (1 - 1e-12):
                st = be.step(min(dt, t_end - t))
                t, n = st["time_seconds"], n + 1
                if adaptive:
                    dt = st["suggested_next_dt"]
            assert steps[i] == n
            assert np.abs(batch.copy_field(i) - be.copy_field(_abi.OBSERVABLE_M)).max() < 1e-6
            be.close()
        batch.close()
