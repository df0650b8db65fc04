"""Brown thermal field on the GPU against the FP64 oracle (crates/fullmag-engine/src/
fdm_fields.rs:818-896): the SplitMix64 counter stream is reproduced with integer
arithmetic and the Box-Muller transform in FP32, so H_eff matches the oracle's noise cell
by cell; trajectories of each fixed-step integrator and of DP45 follow the oracle's, and
the noise changes with the step counter and the step size as the oracle's does."""
import math

import numpy as np
import pytest

from fullmag_gb300 import FdmBackend, _abi
from helpers import problem, rel_l2
from test_gpu_parity import make_pair

pytestmark = pytest.mark.gpu


def test_heff_matches_the_oracle_noise(gpu_lib, oracle):
    kw = problem(40, 24, 3, seed=111, alpha=0.1, temperature=300.0)
    mask = (np.random.default_rng(8).random(40 * 24 * 3) > 0.1).astype(np.uint8)
    gpu, orc = make_pair(oracle, kw, mask=mask)
    m = kw["m0"] * mask[:, None]
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), orc.fields(m)["h_eff"]) < 1e-5
    st, ost = gpu.stats(), orc.observe()
    # the noise enters no energy, and the largest |H_eff| sees it
    assert abs(st["total_energy_joules"] - ost["e_total"]) <= 1e-5 * abs(ost["e_total"])
    assert abs(st["max_effective_field_amplitude"] - ost["max_h_eff"]) <= 1e-5 * ost["max_h_eff"]


def test_noise_statistics(gpu_lib):
    nx, ny, nz = 128, 64, 8
    kw = problem(nx, ny, nz, seed=112, alpha=0.2, b_mt=None, a_ex=0.0, enable_demag=False)
    cold = FdmBackend(**kw).copy_field(_abi.OBSERVABLE_H_EFF)
    hot = FdmBackend(**kw, temperature=100.0).copy_field(_abi.OBSERVABLE_H_EFF)
    g0 = kw["gamma"] * (1 + kw["alpha"] ** 2)
    sig = math.sqrt(2 * kw["alpha"] * 1.380649e-23 * 100.0 /
                    (g0 * 1.2566370614359173e-6 * kw["ms"] * kw["dx"] * kw["dy"] * kw["dz"] * 1e-13))
    z = ((hot - cold) / sig).reshape(-1)
    n = z.size
    assert abs(z.mean()) < 5.0 / math.sqrt(n)
    assert abs(z.std() - 1.0) < 0.01
    assert abs((z ** 4).mean() - 3.0) < 5.0 * math.sqrt(96.0 / n)


@pytest.mark.parametrize("integrator", [_abi.INTEGRATOR_HEUN, _abi.INTEGRATOR_RK4, _abi.INTEGRATOR_ABM3])
def test_trajectory(gpu_lib, oracle, integrator):
    kw = problem(24, 12, 2, seed=113, alpha=0.1, temperature=30.0)
    gpu, orc = make_pair(oracle, kw, integrator=integrator)
    for k in range(20):
        dt = 5e-14 if k < 12 else 4e-14  # a change of dt changes the amplitude
        sg = gpu.step(dt)
        so = orc.step(dt)
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 2e-5
    assert abs(sg["max_rhs_amplitude"] - so["max_rhs"]) <= 1e-4 * so["max_rhs"]
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), orc.fields(orc.get_m())["h_eff"]) < 1e-5


def test_dp45_trajectory(gpu_lib, oracle):
    kw = problem(24, 12, 2, seed=114, alpha=0.1, temperature=10.0, adaptive_max_error=1e-4)
    gpu, orc = make_pair(oracle, kw, integrator=_abi.INTEGRATOR_DP45)
    dt = 2e-14
    for _ in range(10):
        sg = gpu.step(dt)
        so = orc.step(dt)
        # a rejected attempt retries at a size from each side's own error estimate (FP32 on
        # the GPU), so the times drift apart slightly; |dm/dt| dt_diff stays below 1e-5
        assert abs(sg["time_seconds"] - so["time"]) <= 1e-4 * so["time"]
        dt = so["suggested_next_dt"]
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 1e-4
    # an observable read between steps keeps the first-same-as-last derivative
    gpu.copy_field(_abi.OBSERVABLE_H_EFF)
    orc.fields(orc.get_m())
    gpu.step(dt)
    orc.step(dt)
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 1e-4


def test_step_many_advances_the_counter(gpu_lib, oracle):
    kw = problem(16, 8, 2, seed=115, alpha=0.1, temperature=30.0)
    gpu, orc = make_pair(oracle, kw, integrator=_abi.INTEGRATOR_RK4)
    gpu.step_many(5e-14, 6)
    for _ in range(6):
        orc.step(5e-14)
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 2e-5


def test_batch_matches_single_runs(gpu_lib):
    # problems with extra-field terms take the batch driver's per-problem path; the thermal
    # counter, the amplitude's dt (the last step is cut to t_end) and the DP45 retries must
    # come out as in single-problem stepping
    from fullmag_gb300 import FdmBatch
    reg = (np.arange(20 * 10 * 2) % 2).astype(np.uint32)
    ps = [problem(20, 10, 2, seed=116, alpha=0.1, temperature=30.0, region_mask=reg),
          problem(16, 8, 1, seed=117, alpha=0.1, temperature=10.0, adaptive_max_error=1e-4)]
    ps[0]["integrator"] = _abi.INTEGRATOR_RK4
    ps[1]["integrator"] = _abi.INTEGRATOR_DP45
    t_end, dt0 = 6.3e-13, 5e-14
    batch = FdmBatch(ps)
    steps, _ = batch.step_until(t_end, dt0)
    for i, kw in enumerate(ps):
        be = FdmBackend(**kw)
        t, dt, n = 0.0, dt0, 0
        while t < t_end * (1 - 1e-12):
            st = be.step(min(dt, t_end - t))
            t, n = st["time_seconds"], n + 1
            if kw["integrator"] == _abi.INTEGRATOR_DP45:
                dt = st["suggested_next_dt"]
        assert steps[i] == n
        assert np.abs(batch.copy_field(i) - be.copy_field(_abi.OBSERVABLE_M)).max() < 1e-6
        be.close()
    batch.close()
