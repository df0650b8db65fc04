"""Batched sweep (fullmag_fdm_batch_*): problems of uneven size advanced together must
follow exactly the trajectories they follow alone through fullmag_fdm_backend_step."""
import numpy as np
import pytest

from fullmag_gb300 import FdmBackend, FdmBatch, FdmError, _abi
from helpers import problem

pytestmark = pytest.mark.gpu


def plans():
    out = []
    for i, (nx, ny, nz) in enumerate([(17, 9, 1), (24, 16, 2), (12, 20, 4), (33, 5, 1)]):
        kw = problem(nx, ny, nz, seed=40 + i, alpha=0.05 + 0.02 * i, b_mt=(20.0 * i, 10.0, 0.0))
        kw["integrator"] = _abi.INTEGRATOR_DP45
        kw["adaptive_max_error"] = 1e-5
        out.append(kw)
    return out


def run_alone(kw, t_end, dt0):
    be = FdmBackend(**kw)
    t, dt, n = 0.0, dt0, 0
    while t < t_end * (1 - 1e-12):
        st = be.step(min(dt, t_end - t))
        t, dt, n = st["time_seconds"], st["suggested_next_dt"], n + 1
    m = be.copy_field(_abi.OBSERVABLE_M)
    be.close()
    return m, n


def test_batch_matches_single_problems(gpu_lib):
    ps = plans()
    batch = FdmBatch(ps)
    assert len(batch) == 4
    t_end, dt0 = 2e-12, 1e-13
    steps, wall = batch.step_until(t_end, dt0)
    for i, kw in enumerate(ps):
        m_alone, n_alone = run_alone(kw, t_end, dt0)
        assert steps[i] == n_alone
        assert abs(batch.stats(i)["time_seconds"] - t_end) < 1e-24
        assert np.abs(batch.copy_field(i) - m_alone).max() < 1e-6
        assert wall[i] > 0
    # continuing carries each problem's own step size
    steps2, _ = batch.step_until(3e-12, dt0)
    assert all(s >= 1 for s in steps2)
    batch.close()


def test_batch_fixed_step(gpu_lib):
    ps = []
    for i, (nx, ny, nz) in enumerate([(16, 8, 2), (10, 10, 1)]):
        kw = problem(nx, ny, nz, seed=60 + i)
        kw["integrator"] = _abi.INTEGRATOR_RK4
        ps.append(kw)
    batch = FdmBatch(ps)
    steps, _ = batch.step_until(1e-12, 5e-14)
    assert list(steps) == [20, 20]
    for i, kw in enumerate(ps):
        be = FdmBackend(**kw)
        for _ in range(20):
            be.step(5e-14)
        assert np.abs(batch.copy_field(i) - be.copy_field(_abi.OBSERVABLE_M)).max() < 1e-6


def test_batch_reports_bad_plan(gpu_lib):
    ps = plans()[:2]
    ps[1] = dict(ps[1], m0=ps[1]["m0"][:-1])
    with pytest.raises(FdmError, match="problem 1"):
        FdmBatch(ps)
