"""The reference's benchmark configurations at their own sizes, CUDA engine vs the FP64
oracle, through the C ABI, with the demag tensor built by the engine itself (FP64 Newell
setup on the GPU, no spectra passed in).

- GPU Newell builder vs the oracle's restatement of newell.rs on grids whose extents pass
  the 40-cell asymptotic threshold (crates/fullmag-fdm-demag/src/newell.rs:212-229,
  254-519), so both the 27-point f/g stencil at large arguments (where f and g cancel)
  and the dipole asymptotics are exercised: H_demag within 1e-5 relative L2.
- The 256x256x64 RK4 volume (the roofline configuration): H_eff within 1e-5 relative L2
  at steps 0, 1, 2, 5 and 10.
- The 512x128x1 Dormand-Prince film: H_eff at t = 0 within 1e-5; at least 200 adaptive
  steps, each side with its own step controller to the same end time; the time averages
  of <m> and of the energies over the run within 1e-4 relative (the FP32 state and the
  FP32 error norm make the two controllers pick slightly different steps).
"""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

from fullmag_gb300 import FdmBackend, _abi
from helpers import problem, rel_l2

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
HEFF_TOL = 1e-5


def _bench():
    if str(ROOT) not in sys.path:
        sys.path.insert(0, str(ROOT))
    import bench
    return bench


def _oracle_for(oracle, kw, integrator, **extra):
    oint = {_abi.INTEGRATOR_HEUN: oracle.HEUN, _abi.INTEGRATOR_RK4: oracle.RK4,
            _abi.INTEGRATOR_DP45: oracle.DP45}[integrator]
    okw = {k: v for k, v in kw.items() if k != "adaptive_max_error"}
    oracle.set_threads(os.cpu_count() or 1)
    return oracle.Problem(**okw, integrator=oint, **extra)


@pytest.mark.parametrize("grid,d", [((96, 64, 48), (2e-9, 2.5e-9, 3e-9)),
                                    ((512, 128, 1), (3.90625e-9, 3.90625e-9, 3e-9)),
                                    ((160, 48, 4), (3e-9, 3e-9, 1e-9))])
def test_gpu_newell_demag_vs_oracle(gpu_lib, oracle, grid, d):
    nx, ny, nz = grid
    kw = problem(nx, ny, nz, d=d, seed=11, b_mt=None, enable_exchange=False)
    gpu = FdmBackend(**kw, integrator=_abi.INTEGRATOR_RK4)  # tensor built on the GPU in FP64
    orc = _oracle_for(oracle, kw, _abi.INTEGRATOR_RK4)
    h_ref = orc.fields()["h_demag"]
    err = rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_DEMAG), h_ref)
    gpu.close()
    orc.close()
    assert err < HEFF_TOL, err


def test_volume_256x256x64_rk4_heff_over_steps(gpu_lib, oracle):
    b = _bench()
    w = b.WORKLOADS["volume_256x256x64_rk4"]
    kw, integ = b.gpu_plan(w)
    gpu = FdmBackend(**kw, integrator=integ)
    orc = _oracle_for(oracle, kw, integ)
    errs = {}
    done = 0
    for s in (0, 1, 2, 5, 10):
        while done < s:
            gpu.step(w["dt"])
            orc.step(w["dt"])
            done += 1
        errs[s] = rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), orc.fields()["h_eff"])
    gpu.close()
    orc.close()
    print("H_eff rel L2 by step:", errs)
    assert all(e < HEFF_TOL for e in errs.values()), errs


def _run_to(be, t_end, dt0, is_gpu):
    """Adaptive steps to t_end: time, <m>, total energy and exchange energy after each
    accepted step (the initial state first)."""
    rows = []
    t, dt = 0.0, dt0

    def record(t, st):
        m = be.copy_field(_abi.OBSERVABLE_M) if is_gpu else be.get_m()
        if is_gpu:
            e = (st["total_energy_joules"], st["exchange_energy_joules"], st["demag_energy_joules"])
        else:
            e = (st["e_total"], st["e_exchange"], st["e_demag"])
        rows.append((t, *m.mean(axis=0), *e))

    record(0.0, be.stats() if is_gpu else be.observe())
    while t < t_end * (1 - 1e-12):
        st = be.step(min(dt, t_end - t))
        t = st["time_seconds"] if is_gpu else st["time"]
        dt = st["suggested_next_dt"]
        record(t, st)
    return np.array(rows)


def _time_average(rows):
    t, v = rows[:, 0], rows[:, 1:]
    area = (0.5 * (v[1:] + v[:-1]) * np.diff(t)[:, None]).sum(axis=0)
    return area / (t[-1] - t[0])


def test_film_512x128x1_dp45_vs_oracle(gpu_lib, oracle):
    b = _bench()
    w = b.WORKLOADS["film_512x128x1_dp45"]
    kw, integ = b.gpu_plan(w)
    gpu = FdmBackend(**kw, integrator=integ)
    assert gpu.fft_shape()[0] == 1024  # x half-length 512: the row pass's general transform
    orc = _oracle_for(oracle, kw, integ, max_error=w["max_error"])
    err0 = rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), orc.fields()["h_eff"])
    assert err0 < HEFF_TOL, err0
    t_end = 65e-12
    rg = _run_to(gpu, t_end, w["dt"], True)
    ro = _run_to(orc, t_end, w["dt"], False)
    gpu.close()
    orc.close()
    assert len(rg) - 1 >= 200, len(rg)
    ag, ao = _time_average(rg), _time_average(ro)
    # <m> components: absolute (|<m>| <= 1); energies: relative
    assert np.abs(ag[:3] - ao[:3]).max() < 1e-4, (ag[:3], ao[:3])
    for k in range(3, 6):
        assert abs(ag[k] - ao[k]) <= 1e-4 * abs(ao[k]), (k, ag[k], ao[k])
    # and the states at the common end time
    assert np.abs(rg[-1, 1:4] - ro[-1, 1:4]).max() < 1e-4
