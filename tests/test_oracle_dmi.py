"""DMI and magnetoelastic terms of the oracle (native/backends/fdm/src/demag_fp32.cu:319-376,
reductions_fp64.cu:647-720): known answers for a uniform state, a helix and a single
strain component, and the energy conventions the reference reports."""
import numpy as np

from helpers import MU0, problem, random_unit

D_INT, D_BULK = 3e-3, 2e-3


def _no_demag(nx, ny, nz, m0, **extra):
    kw = problem(nx, ny, nz, seed=1, b_mt=None)
    kw["m0"] = m0
    kw["enable_demag"] = False
    kw["a_ex"] = 0.0
    kw.update(extra)
    return kw


def test_uniform_state_has_no_dmi(oracle):
    m = np.tile([0.6, 0.0, 0.8], (5 * 4 * 3, 1))
    pr = oracle.Problem(**_no_demag(5, 4, 3, m, dmi_d_interfacial=D_INT, dmi_d_bulk=D_BULK))
    assert np.abs(pr.fields()["h_eff"]).max() < 1e-9
    assert abs(pr.observe()["e_dmi"]) < 1e-30


def test_interfacial_helix_central_differences(oracle):
    """m = (cos kx, 0, sin kx) along a chain: H_x = 2D/(mu0 Ms) (m_z(x+d) - m_z(x-d)) / 2d,
    H_z = -2D/(mu0 Ms) (m_x(x+d) - m_x(x-d)) / 2d, one-sided at the clamped ends."""
    nx, d, ms = 16, 2e-9, 8e5
    k = 2 * np.pi / (nx * d)
    x = np.arange(nx) * d
    m = np.stack([np.cos(k * x), np.zeros(nx), np.sin(k * x)], axis=1)
    kw = _no_demag(nx, 1, 1, m, dmi_d_interfacial=D_INT)
    kw.update(dx=d, dy=d, dz=d, ms=ms)
    h = oracle.Problem(**kw).fields()["h_eff"]
    xm = np.maximum(np.arange(nx) - 1, 0)
    xp = np.minimum(np.arange(nx) + 1, nx - 1)
    pf = 2 * D_INT / (MU0 * ms)
    want_x = pf * (m[xp, 2] - m[xm, 2]) / (2 * d)
    want_z = -pf * (m[xp, 0] - m[xm, 0]) / (2 * d)
    assert np.allclose(h[:, 0], want_x, rtol=1e-12, atol=1e-6)
    assert np.allclose(h[:, 2], want_z, rtol=1e-12, atol=1e-6)
    assert np.abs(h[:, 1]).max() < 1e-9


def test_dmi_energy_conventions(oracle):
    """Interfacial: E = -1/2 mu0 Ms V sum m.H_dmi.  Bulk: the reference reports
    +V D sum m.(curl m) while its field is +2D/(mu0 Ms) curl m, i.e. E = +1/2 mu0 Ms V
    sum m.H_dmi; the oracle keeps both as the reference has them."""
    n = 6 * 5 * 3
    m = random_unit(n, 7)
    mask = np.ones(n, dtype=np.uint8)
    mask[[3, 17, 40]] = 0
    for key, sign in (("dmi_d_interfacial", -0.5), ("dmi_d_bulk", +0.5)):
        kw = _no_demag(6, 5, 3, m, **{key: 2.5e-3})
        pr = oracle.Problem(**kw, active_mask=mask)
        h = pr.fields()["h_eff"]
        st = pr.observe()
        V = kw["dx"] * kw["dy"] * kw["dz"]
        mm = pr.get_m()
        want = sign * MU0 * kw["ms"] * V * float(np.sum(mm * h))
        assert np.isclose(st["e_dmi"], want, rtol=1e-10), key
        assert np.isclose(st["e_total"], st["e_dmi"], rtol=1e-12)  # no other term is on


def test_magnetoelastic_field(oracle):
    n = 4 * 3 * 2
    m = random_unit(n, 8)
    strain = (1e-3, -2e-4, 3e-4, 4e-4, -6e-4, 8e-4)  # Voigt: e11 e22 e33 2e23 2e13 2e12
    b1, b2, ms = 5e6, 7e6, 8e5
    kw = _no_demag(4, 3, 2, m, mel_b1=b1, mel_b2=b2, mel_strain=strain)
    kw["ms"] = ms
    h = oracle.Problem(**kw).fields()["h_eff"]
    e11, e22, e33 = strain[:3]
    e23, e13, e12 = (0.5 * s for s in strain[3:])
    a = -1.0 / (MU0 * ms)
    want = np.stack([
        a * (2 * b1 * m[:, 0] * e11 + b2 * (m[:, 1] * e12 + m[:, 2] * e13)),
        a * (2 * b1 * m[:, 1] * e22 + b2 * (m[:, 0] * e12 + m[:, 2] * e23)),
        a * (2 * b1 * m[:, 2] * e33 + b2 * (m[:, 0] * e13 + m[:, 1] * e23))], axis=1)
    assert np.allclose(h, want, rtol=1e-12, atol=1e-9)
