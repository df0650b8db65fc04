"""Spin-transfer and spin-orbit torques of the oracle (native/backends/fdm/src/llg_fp32.cu:65-195,
prefactors api.cpp:250-300 and context.hpp:321-339): closed forms on field-free states
and a numpy restatement of the upwind Zhang-Li derivative."""
import numpy as np

from helpers import MU0, problem, random_unit

HBAR, E_CH, MU_B = 1.054571817e-34, 1.60217662e-19, 9.274009994e-24


def _bare(nx, ny, nz, m, **extra):
    kw = problem(nx, ny, nz, seed=1, b_mt=None, alpha=0.1)
    kw.update(m0=m, enable_demag=False, a_ex=0.0)
    kw.update(extra)
    return kw


def test_sot_closed_form(oracle):
    n = 4 * 3 * 2
    m = random_unit(n, 11)
    sigma = np.array([0.0, 2.0, 1.0])
    je, xi_dl, xi_fl, t = 2e11, 0.3, -0.1, 2e-9
    kw = _bare(4, 3, 2, m, sot_je=je, sot_xi_dl=xi_dl, sot_xi_fl=xi_fl, sot_sigma=tuple(sigma), sot_thickness=t)
    rhs = oracle.Problem(**kw).fields()["rhs"]
    s = sigma / np.linalg.norm(sigma)
    amp = abs(je) * HBAR / (2 * E_CH * MU0 * kw["ms"] * t)
    ms_ = m @ s
    want = amp * (-xi_dl * (ms_[:, None] * m - s) + xi_fl * np.cross(m, s))
    assert np.allclose(rhs, want, rtol=1e-12, atol=1e-9 * np.abs(want).max())


def test_slonczewski_closed_form(oracle):
    n = 5 * 2 * 1
    m = random_unit(n, 12)
    p = np.array([0.3, -0.2, 0.9])
    lam, eps, P, j = 2.0, 0.15, 0.6, np.array([0.0, 0.0, 3e11])
    kw = _bare(5, 2, 1, m, current_density=tuple(j), stt_p=tuple(p), stt_lambda=lam, stt_epsilon_prime=eps,
               stt_degree=P)
    # Zhang-Li is on as well (stt_degree > 0, j != 0) but vanishes along z for a single layer
    rhs = oracle.Problem(**kw).fields()["rhs"]
    pf = np.linalg.norm(j) * HBAR / (2 * E_CH * MU0 * kw["ms"] * kw["dz"])
    L2 = lam * lam
    g = P * L2 / ((L2 + 1) + (L2 - 1) * (m @ p))
    mxp = np.cross(m, p)
    want = (pf * g)[:, None] * (np.cross(m, mxp) + eps * mxp)
    assert np.allclose(rhs, want, rtol=1e-12, atol=1e-9 * np.abs(want).max())


def test_zhang_li_upwind(oracle):
    """Uniform state: no torque.  Helix along x with u_x > 0: D = u_x (m_i - m_{i-1}) / dx
    (none at x = 0), torque -m x (m x D) - beta m x D."""
    nx, d = 12, 3e-9
    uni = np.tile([0.0, 0.6, 0.8], (nx, 1))
    j = (4e11, 0.0, 0.0)
    P, beta = 0.5, 0.04
    kw = _bare(nx, 1, 1, uni, current_density=j, stt_degree=P, stt_beta=beta, dx=d, dy=d, dz=d)
    assert np.abs(oracle.Problem(**kw).fields()["rhs"]).max() < 1e-9
    k = 2 * np.pi / (nx * d)
    x = np.arange(nx) * d
    m = np.stack([np.cos(k * x), np.sin(k * x), np.zeros(nx)], axis=1)
    kw["m0"] = m
    rhs = oracle.Problem(**kw).fields()["rhs"]
    u = P * MU_B / (E_CH * kw["ms"] * (1 + beta * beta)) * j[0]
    D = np.zeros_like(m)
    D[1:] = u * (m[1:] - m[:-1]) / d
    c1 = np.cross(m, D)
    want = -np.cross(m, c1) - beta * c1
    assert np.allclose(rhs, want, rtol=1e-10, atol=1e-9 * np.abs(want).max())
