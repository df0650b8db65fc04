"""Oersted field of a cylindrical conductor in the oracle (native/backends/fdm/src/context.cu:844-905,
demag_fp32.cu:585-616): H_phi = I r / (2 pi R^2) inside, I / (2 pi r) outside, around z,
scaled by the current's time dependence."""
import numpy as np
import pytest

from helpers import problem


def _kw(**extra):
    kw = problem(10, 8, 1, seed=1, b_mt=None, alpha=0.1)
    kw.update(enable_demag=False, a_ex=0.0)
    kw.update(extra)
    return kw


def _expected(kw, I, R, cx, cy):
    nx, ny, d = kw["nx"], kw["ny"], kw["dx"]
    out = np.zeros((nx * ny, 3))
    for i in range(nx * ny):
        x, y = (i % nx + 0.5) * d - cx, (i // nx + 0.5) * d - cy
        r = np.hypot(x, y)
        hphi = I * r / (2 * np.pi * R * R) if r < R else I / (2 * np.pi * r)
        out[i] = (-hphi * y / r, hphi * x / r, 0.0)
    return out


def test_dc_field_inside_and_outside(oracle):
    R, cx, cy, I = 12e-9, 17e-9, 13e-9, 2.5e-3
    kw = _kw(oersted_current=I, oersted_radius=R, oersted_center=(cx, cy, 0.0))
    h = oracle.Problem(**kw).fields()["h_eff"]
    want = _expected(kw, I, R, cx, cy)
    assert np.allclose(h, want, rtol=1e-12, atol=1e-9 * np.abs(want).max())
    assert np.abs(want).max() > 0
    with pytest.raises(ValueError):
        oracle.Problem(**_kw(oersted_current=I, oersted_radius=0.0))


def test_time_dependence(oracle):
    R, cx, cy, I = 10e-9, 20e-9, 16e-9, 1e-3
    f, phase, off = 3e11, 0.4, 0.2
    kw = _kw(oersted_current=I, oersted_radius=R, oersted_center=(cx, cy, 0.0), oersted_kind=1,
             oersted_freq=f, oersted_phase=phase, oersted_offset=off)
    pr = oracle.Problem(**kw)
    unit = _expected(kw, 1.0, R, cx, cy)
    for _ in range(3):
        t = pr.observe()["time"]
        want = unit * I * (np.sin(2 * np.pi * f * t + phase) + off)
        assert np.allclose(pr.fields(pr.get_m())["h_eff"], want, rtol=1e-10, atol=1e-12)
        pr.step(1e-13)
    pulse = _kw(oersted_current=I, oersted_radius=R, oersted_center=(cx, cy, 0.0), oersted_kind=2,
                oersted_t_on=1.5e-13, oersted_t_off=2.5e-13)
    pr = oracle.Problem(**pulse)
    seen = []
    for _ in range(4):
        seen.append(np.abs(pr.fields(pr.get_m())["h_eff"]).max() > 0)
        pr.step(1e-13)
    assert seen == [False, False, True, False]
