"""RK23 (Bogacki-Shampine 3(2) + FSAL) and ABM3 (Adams-Bashforth-Moulton 3) of the oracle,
as the C ABI runs them (native/backends/fdm/src/llg_rk23_fp32.cu:150-265,
native/backends/fdm/src/llg_abm3_fp32.cu:115-266): convergence against a fine RK4
trajectory, ABM3's third order, its Heun start-up and restart on a dt change, and
RK23's step control."""
import numpy as np

from helpers import problem


def _run(oracle, kw, integrator, dt, steps, **extra):
    pr = oracle.Problem(**kw, integrator=integrator, **extra)
    st = None
    for _ in range(steps):
        st = pr.step(dt)
    return pr, st


def test_abm3_converges_with_third_order(oracle):
    kw = problem(6, 5, 2, seed=31, alpha=0.3)
    t_end = 4e-12
    ref, _ = _run(oracle, kw, oracle.RK4, t_end / 800, 800)
    errs = []
    for steps in (80, 160, 320):
        pr, _ = _run(oracle, kw, oracle.ABM3, t_end / steps, steps)
        errs.append(np.abs(pr.get_m() - ref.get_m()).max())
    assert errs[-1] < 5e-6
    # third order: halving dt divides the error by about 8 (Heun start-up steps included)
    assert errs[0] / errs[1] > 5.0 and errs[1] / errs[2] > 5.0, errs


def test_abm3_startup_and_restart_are_heun_steps(oracle):
    kw = problem(5, 4, 2, seed=32)
    dt = 5e-14
    abm = oracle.Problem(**kw, integrator=oracle.ABM3)
    heun = oracle.Problem(**kw, integrator=oracle.HEUN)
    for _ in range(3):  # start-up
        abm.step(dt)
        heun.step(dt)
        assert np.array_equal(abm.get_m(), heun.get_m())
    abm.step(dt)  # first Adams step differs from Heun
    heun.step(dt)
    assert not np.array_equal(abm.get_m(), heun.get_m())
    # a step size change of more than 10 % restarts with Heun steps from the current state
    heun.set_m(abm.get_m())
    abm.step(1.5 * dt)
    heun.step(1.5 * dt)
    assert np.array_equal(abm.get_m(), heun.get_m())
    # a change of 10 % or less keeps the Adams steps going (no restart)
    abm2 = oracle.Problem(**kw, integrator=oracle.ABM3)
    for _ in range(4):
        abm2.step(dt)
    heun.set_m(abm2.get_m())
    abm2.step(1.05 * dt)
    heun.step(1.05 * dt)
    assert not np.array_equal(abm2.get_m(), heun.get_m())


def test_rk23_converges_and_controls_the_step(oracle):
    kw = problem(6, 5, 2, seed=33, alpha=0.3)
    t_end = 4e-12
    ref, _ = _run(oracle, kw, oracle.RK4, t_end / 400, 400)
    pr = oracle.Problem(**kw, integrator=oracle.RK23, max_error=1e-7, dt_max=1e-12)
    t, dt, rejected, steps = 0.0, 1e-13, 0, 0
    while t < t_end * (1 - 1e-12):
        st = pr.step(min(dt, t_end - t))
        t, dt = st["time"], st["suggested_next_dt"]
        rejected += st["rejected_attempts"]
        steps += 1
    assert np.abs(pr.get_m() - ref.get_m()).max() < 1e-5
    assert rejected > 0 and steps > 5
    # from the same state and step, a looser tolerance suggests a larger next step
    sugg = [oracle.Problem(**kw, integrator=oracle.RK23, max_error=tol, dt_max=1e-12).step(1e-14)["suggested_next_dt"]
            for tol in (1e-7, 1e-4)]
    assert sugg[1] > sugg[0]
