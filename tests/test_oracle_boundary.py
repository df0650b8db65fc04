"""The oracle's restatement of the double-precision path's boundary correction against
closed forms (CPU): T0 face-link exchange (native/backends/fdm/src/exchange_t0_fp64.cu),
T1 boundary stencil (exchange_t1_fp64.cu), the phi-weighted demag input and energies
(demag_fp64.cu:55-90, reductions_fp64.cu:123-260) and the sparse demag correction
(demag_boundary_fp64.cu:23-76)."""
import numpy as np
import pytest

from helpers import random_unit

MU0 = 4e-7 * np.pi
MS, A = 8e5, 1.3e-11


def _prob(oracle, nx, ny, nz, d=(2e-9, 2e-9, 2e-9), m0=None, boundary=None, demag=False, exchange=True, seed=3):
    n = nx * ny * nz
    return oracle.Problem(nx=nx, ny=ny, nz=nz, dx=d[0], dy=d[1], dz=d[2], ms=MS, a_ex=A, alpha=0.1,
                          m0=random_unit(n, seed) if m0 is None else m0, enable_demag=demag,
                          enable_exchange=exchange, boundary=boundary)


def test_t0_and_t1_reduce_to_the_standard_exchange_inside(oracle):
    nx, ny, nz, d = 6, 5, 4, (2e-9, 2.5e-9, 3e-9)
    n = nx * ny * nz
    ones = np.ones(n)
    ref = _prob(oracle, nx, ny, nz, d).fields()["h_ex"]
    t0 = _prob(oracle, nx, ny, nz, d, boundary={"tier": 1, "volume_fraction": ones, "face": [ones] * 6}).fields()["h_ex"]
    dl = [np.full(n, d[0])] * 2 + [np.full(n, d[1])] * 2 + [np.full(n, d[2])] * 2
    t1 = _prob(oracle, nx, ny, nz, d, boundary={"tier": 2, "volume_fraction": ones, "delta": dl}).fields()["h_ex"]
    assert np.abs(t0 - ref).max() <= 1e-12 * np.abs(ref).max()
    assert np.abs(t1 - ref).max() <= 1e-12 * np.abs(ref).max()


def test_t0_face_link_closed_form(oracle):
    # two cells along x: cell 0 (phi 0.8) couples to cell 1 through a face of fraction 0.5
    d = (2e-9, 2e-9, 2e-9)
    m0 = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])
    phi = np.array([0.8, 1.0])
    f = [np.zeros(2) for _ in range(6)]
    f[0][0] = 0.5  # +x face of cell 0
    f[1][1] = 0.5  # -x face of cell 1
    h = _prob(oracle, 2, 1, 1, d, m0=m0, boundary={"tier": 1, "volume_fraction": phi, "face": f}).fields()["h_ex"]
    want0 = 2.0 / (MU0 * MS * 0.8) * A * 0.5 * (m0[1] - m0[0]) / d[0] ** 2
    want1 = 2.0 / (MU0 * MS * 1.0) * A * 0.5 * (m0[0] - m0[1]) / d[0] ** 2
    assert np.allclose(h[0], want0, rtol=1e-13, atol=0.0) and np.allclose(h[1], want1, rtol=1e-13, atol=0.0)


def test_t1_boundary_stencil_closed_form(oracle):
    # three cells along x; the boundary sits half a cell beyond the centre of cell 1 on -x,
    # so its +x neighbour couples with 2 A / (dx (dx + delta_-x)); a floor of 0.1 dx
    dx = 2e-9
    m0 = random_unit(3, 7)
    n = 3
    dl = [np.full(n, dx) for _ in range(6)]
    dl[1][1] = 0.5 * dx
    h = _prob(oracle, 3, 1, 1, (dx, dx, dx), m0=m0,
              boundary={"tier": 2, "volume_fraction": np.ones(n), "delta": dl, "delta_min": 0.1 * dx}).fields()["h_ex"]
    s = 2.0 / (MU0 * MS)
    want = s * (A * 2.0 / (dx * (dx + 0.5 * dx)) * (m0[2] - m0[1]) + A * 2.0 / (dx * (dx + dx)) * (m0[0] - m0[1]))
    assert np.allclose(h[1], want, rtol=1e-13, atol=0.0)


def test_phi_weighted_demag_input_and_energy(oracle):
    # a uniform fraction c scales the demag input by c and weights the energy by c: E_d(c) = c^2 E_d(1)
    nx, ny, nz = 6, 4, 3
    n = nx * ny * nz
    c = 0.6
    m0 = random_unit(n, 11)
    e1 = _prob(oracle, nx, ny, nz, m0=m0, demag=True, exchange=False).observe()
    ones = np.ones(n)
    ec = _prob(oracle, nx, ny, nz, m0=m0, demag=True, exchange=False,
               boundary={"tier": 1, "volume_fraction": c * ones, "face": [ones] * 6}).observe()
    assert ec["e_demag"] == pytest.approx(c * c * e1["e_demag"], rel=1e-12)


def test_sparse_demag_correction_is_added_to_the_targets(oracle):
    nx, ny, nz = 5, 4, 2
    n = nx * ny * nz
    m0 = random_unit(n, 5)
    base = _prob(oracle, nx, ny, nz, m0=m0, demag=True, exchange=False).fields()["h_demag"]
    rng = np.random.default_rng(2)
    tgt = np.array([3, 17], dtype=np.int32)
    src = np.array([3, 4, -1, 17, 16, 18], dtype=np.int32)  # stencil 3, one empty slot
    ten = rng.normal(0.0, 0.05, size=(2, 3, 6))
    phi = rng.uniform(0.5, 1.0, n)
    got = _prob(oracle, nx, ny, nz, m0=m0, demag=True, exchange=False,
                boundary={"tier": 0, "volume_fraction": phi, "corr": (tgt, src, ten.reshape(-1))}).fields()["h_demag"]
    want = base.copy()
    for t in range(2):
        for q in range(3):
            s = src[3 * t + q]
            if s < 0:
                continue
            Nxx, Nxy, Nxz, Nyy, Nyz, Nzz = ten[t, q]
            N = np.array([[Nxx, Nxy, Nxz], [Nxy, Nyy, Nyz], [Nxz, Nyz, Nzz]])
            want[tgt[t]] -= N @ (phi[s] * MS * m0[s])
    assert np.allclose(got, want, rtol=1e-12, atol=1e-9 * np.abs(base).max())
