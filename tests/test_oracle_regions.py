"""Inter-region exchange of the oracle (native/backends/fdm/src/exchange_fp32.cu:48-104,
native/backends/fdm/src/api.cpp:405-420): per-cell region ids below 256 and a 256 x 256
stiffness table; without a table A sits on the diagonal and regions decouple.

The field 2/(mu0 Ms) sum_q A[r_i][r_q] (m_q - m_i) / d_q^2 (Neumann clamp: a missing
neighbour is the cell itself) and the pair energy sum A_ij V |m_j - m_i|^2 / d^2 are
restated below with numpy loops on small grids."""
import numpy as np
import pytest

from helpers import MU0, problem


def _regions(nx, ny, nz, seed):
    rng = np.random.default_rng(seed)
    x = np.tile(np.arange(nx), ny * nz)
    reg = np.where(x < nx // 2, 0, 1).astype(np.uint32)
    reg[rng.random(reg.size) < 0.15] = 7
    lut = np.zeros((256, 256))
    lut[0, 0], lut[1, 1], lut[7, 7] = 1.3e-11, 0.7e-11, 2e-11
    lut[0, 1] = lut[1, 0] = 0.3e-11
    lut[1, 7] = lut[7, 1] = 0.5e-11
    return reg, lut


def _restated(kw, reg, lut):
    nx, ny, nz = kw["nx"], kw["ny"], kw["nz"]
    d = (kw["dx"], kw["dy"], kw["dz"])
    m = kw["m0"].reshape(nz, ny, nx, 3)
    r = reg.reshape(nz, ny, nx)
    s = 2.0 / (MU0 * kw["ms"])
    h = np.zeros_like(m)
    e = 0.0
    V = d[0] * d[1] * d[2]
    for z in range(nz):
        for y in range(ny):
            for x in range(nx):
                for ax, (dz_, dy_, dx_) in enumerate(((0, 0, 1), (0, 1, 0), (1, 0, 0))):
                    for sgn in (-1, 1):
                        zz, yy, xx = z + sgn * dz_, y + sgn * dy_, x + sgn * dx_
                        if not (0 <= zz < nz and 0 <= yy < ny and 0 <= xx < nx):
                            continue  # clamped neighbour: m_q - m_i = 0
                        a = lut[r[z, y, x], r[zz, yy, xx]]
                        dm = m[zz, yy, xx] - m[z, y, x]
                        h[z, y, x] += s * a * dm / d[ax] ** 2
                        if sgn == 1:
                            e += a * V * np.dot(dm, dm) / d[ax] ** 2
    return h.reshape(-1, 3), e


@pytest.mark.parametrize("with_table", [True, False])
def test_region_exchange_field_and_energy(oracle, with_table):
    reg, lut = _regions(6, 5, 3, seed=3)
    kw = problem(6, 5, 3, seed=15)
    table = lut if with_table else None
    pr = oracle.Problem(**kw, enable_demag=False, region_mask=reg, exchange_lut=table)
    if not with_table:
        lut = np.zeros((256, 256))
        lut[np.arange(256), np.arange(256)] = kw["a_ex"]
    want_h, want_e = _restated(kw, reg, lut)
    got = pr.fields()["h_ex"]
    assert np.abs(got - want_h).max() <= 1e-12 * np.abs(want_h).max()
    assert np.isclose(pr.observe()["e_exchange"], want_e, rtol=1e-12)


def test_single_region_matches_uniform_exchange(oracle):
    kw = problem(7, 4, 2, seed=8)
    reg = np.full(7 * 4 * 2, 5, dtype=np.uint32)
    lut = np.zeros((256, 256))
    lut[5, 5] = kw["a_ex"]
    a = oracle.Problem(**kw, region_mask=reg, exchange_lut=lut)
    b = oracle.Problem(**kw)
    fa, fb = a.fields(), b.fields()
    for k in ("h_ex", "h_eff", "rhs"):
        assert np.allclose(fa[k], fb[k], rtol=1e-12, atol=1e-12 * np.abs(fb[k]).max())
    assert np.isclose(a.observe()["e_exchange"], b.observe()["e_exchange"], rtol=1e-12)


def test_region_inputs_are_checked(oracle):
    kw = problem(4, 3, 1, seed=2)
    reg = np.zeros(12, dtype=np.uint32)
    bad = reg.copy()
    bad[3] = 256
    with pytest.raises(ValueError):
        oracle.Problem(**kw, region_mask=bad)
    with pytest.raises(ValueError):
        oracle.Problem(**kw, region_mask=reg[:-1])
    with pytest.raises(ValueError):
        oracle.Problem(**kw, region_mask=reg, exchange_lut=np.zeros(255 * 255))
