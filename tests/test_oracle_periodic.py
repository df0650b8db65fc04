"""The oracle's periodic boundaries (CPU) against the reference CPU engine's definition:
the truncated image-sum tensor folded from the open tensor of the extended grid
(crates/fullmag-engine/src/fdm_fft.rs:614-717, restated here in numpy), the unpadded
FFT convolution against a direct real-space image sum, wrap-around exchange
(fdm_fields.rs:109-160) on a spin wave that is an eigenvector of the periodic
Laplacian, the thin-film limits of the periodic demag field, and the wrapped DMI and
Zhang-Li stencils against numpy restatements."""
import numpy as np
import pytest

from helpers import random_unit

MU0 = 4e-7 * np.pi
MS, A = 8e5, 1.3e-11


def _fold_like_reference(oracle, nx, ny, nz, d, periodic, images):
    """compute_periodic_newell_kernels: the open tensor on the extended grid
    n (1 + 2 I), folded image by image (z, y, x outer to inner) onto the (p_x, p_y, p_z)
    grid, p = n periodic, 2n open."""
    I = [images[a] if periodic[a] else 0 for a in range(3)]
    en = [n * (1 + 2 * i) for n, i in zip((nx, ny, nz), I)]
    kopen = oracle.newell_kernels(en[0], en[1], en[2], *d)  # (6, 2 enz, 2 eny, 2 enx)
    ep = [2 * e for e in en]
    pd = [n if per else 2 * n for n, per in zip((nx, ny, nz), periodic)]
    out = np.zeros((6, pd[2], pd[1], pd[0]))
    for k in range(pd[2]):
        for j in range(pd[1]):
            for i in range(pd[0]):
                acc = np.zeros(6)
                for mz in range(-I[2], I[2] + 1):
                    for my in range(-I[1], I[1] + 1):
                        for mx in range(-I[0], I[0] + 1):
                            ei = (i + mx * nx) % ep[0]
                            ej = (j + my * ny) % ep[1]
                            ek = (k + mz * nz) % ep[2]
                            acc += kopen[:, ek, ej, ei]
                out[:, k, j, i] = acc
    return out


@pytest.mark.parametrize("shape,periodic,images", [
    ((4, 3, 2), (1, 1, 0), (2, 1, 0)),
    ((3, 2, 2), (0, 0, 1), (0, 0, 3)),
    ((2, 3, 1), (1, 1, 1), (1, 2, 2)),
    ((5, 1, 1), (1, 0, 0), (0, 0, 0)),
])
def test_image_sum_tensor_matches_the_reference_fold(oracle, shape, periodic, images):
    nx, ny, nz = shape
    d = (3e-9, 2e-9, 4e-9)
    got = oracle.periodic_newell_kernels(nx, ny, nz, *d, periodic, images)
    want = _fold_like_reference(oracle, nx, ny, nz, d, periodic, images)
    scale = np.abs(want).max()
    # the same open values summed in the same order; only the summation's last bit may move
    assert np.abs(got - want).max() <= 1e-14 * scale


def test_image_sum_tensor_is_not_symmetric_under_wrap(oracle):
    # index n - j stands for the offsets n - j + m n, not -j + m n: the truncated sum differs
    # from its mirror by the two tail images, so its spectrum is complex (why the engine
    # carries a complex kernel on periodic grids)
    k = oracle.periodic_newell_kernels(6, 1, 1, 2e-9, 2e-9, 2e-9, (1, 0, 0), (1, 0, 0))
    xx = k[0, 0, 0]
    assert abs(xx[1] - xx[5]) > 1e-6 * abs(xx).max()
    spec = np.fft.fft(xx)
    assert np.abs(spec.imag).max() > 1e-8 * np.abs(spec).max()


@pytest.mark.parametrize("shape,periodic,images", [
    ((6, 4, 2), (1, 1, 0), (2, 2, 0)),
    ((4, 5, 3), (0, 1, 1), (0, 1, 2)),
    ((8, 3, 1), (1, 0, 0), (3, 0, 0)),
    ((4, 4, 1), (1, 1, 1), (2, 2, 4)),
])
def test_fft_demag_equals_direct_image_sum(oracle, shape, periodic, images):
    nx, ny, nz = shape
    n = nx * ny * nz
    rng = np.random.default_rng(n)
    mask = (rng.random(n) > 0.2).astype(np.uint8)
    pr = oracle.Problem(nx=nx, ny=ny, nz=nz, dx=4e-9, dy=3e-9, dz=2e-9, ms=MS, a_ex=A, alpha=0.5,
                        m0=random_unit(n, 3), active_mask=mask, periodic=periodic, image_counts=images)
    hd = pr.fields()["h_demag"]
    ref = pr.demag_direct()
    assert np.abs(hd - ref).max() <= 1e-11 * np.abs(ref).max()


def test_periodic_exchange_spin_wave_is_an_eigenvector(oracle):
    # m = (cos kx, sin kx, 0) with k = 2 pi / (nx dx): the wrapped discrete Laplacian gives
    # exactly (2 cos(k dx) - 2) / dx^2 m at every cell, the first and last included
    nx, ny, nz, d = 12, 3, 2, 2e-9
    x = np.tile(np.arange(nx), ny * nz)
    th = 2 * np.pi * x / nx
    m = np.stack([np.cos(th), np.sin(th), np.zeros_like(th)], axis=1)
    pr = oracle.Problem(nx=nx, ny=ny, nz=nz, dx=d, dy=d, dz=d, ms=MS, a_ex=A, alpha=0.5, m0=m,
                        enable_demag=False, periodic=(1, 0, 0))
    h = pr.fields()["h_ex"]
    lam = 2 * A / (MU0 * MS) * (2 * np.cos(2 * np.pi / nx) - 2) / d ** 2
    assert np.allclose(h, lam * m, rtol=1e-12, atol=1e-12 * abs(lam))
    # open boundaries clamp the ends instead: the end cells differ
    h_open = oracle.Problem(nx=nx, ny=ny, nz=nz, dx=d, dy=d, dz=d, ms=MS, a_ex=A, alpha=0.5, m0=m,
                            enable_demag=False).fields()["h_ex"]
    assert not np.allclose(h_open, lam * m, rtol=1e-6)


def test_periodic_exchange_energy_forms_agree(oracle):
    # the forward-pair sum (wrap pairs included) equals -1/2 mu0 Ms V sum m.H_ex for unit m
    nx, ny, nz = 6, 5, 4
    n = nx * ny * nz
    for per in [(1, 0, 0), (0, 1, 1), (1, 1, 1)]:
        st = oracle.Problem(nx=nx, ny=ny, nz=nz, dx=2e-9, dy=3e-9, dz=2.5e-9, ms=MS, a_ex=A, alpha=0.5,
                            m0=random_unit(n, 9), enable_demag=False, periodic=per).observe()
        assert st["e_exchange"] == pytest.approx(st["e_exchange_field"], rel=1e-12)


def test_periodic_film_limits(oracle):
    # a film periodic in x and y: uniform in-plane m sees almost no field, uniform
    # out-of-plane m almost -Ms (an infinite sheet), to within the truncation of 10 images
    nx, ny = 8, 8
    n = nx * ny
    kw = dict(nx=nx, ny=ny, nz=1, dx=4e-9, dy=4e-9, dz=2e-9, ms=MS, a_ex=A, alpha=0.5, enable_exchange=False,
              periodic=(1, 1, 0))
    h_in = oracle.Problem(m0=np.tile([1.0, 0.0, 0.0], (n, 1)), **kw).fields()["h_demag"]
    h_out = oracle.Problem(m0=np.tile([0.0, 0.0, 1.0], (n, 1)), **kw).fields()["h_demag"]
    assert np.abs(h_in).max() < 0.01 * MS
    assert np.allclose(h_out[:, 2], -MS, rtol=0.01)
    assert np.abs(h_out[:, :2]).max() < 1e-6 * MS


def _grid_fields(nx, ny, nz, arr):
    """(n, 3) x-fastest -> (3, nz, ny, nx)."""
    return arr.reshape(nz, ny, nx, 3).transpose(3, 0, 1, 2)


def test_periodic_interfacial_dmi_wraps(oracle):
    # central differences with the wrapped neighbour on periodic axes
    # (interfacial_dmi_field, fdm_fields.rs:356-392); exchange, demag and Zeeman off so that
    # H_eff is the DMI field alone
    nx, ny, nz, d, D = 6, 5, 2, (2e-9, 3e-9, 2e-9), 3e-3
    n = nx * ny * nz
    m = random_unit(n, 21)
    pr = oracle.Problem(nx=nx, ny=ny, nz=nz, dx=d[0], dy=d[1], dz=d[2], ms=MS, a_ex=A, alpha=0.5, m0=m,
                        enable_exchange=False, enable_demag=False, dmi_d_interfacial=D, periodic=(1, 1, 0))
    h = _grid_fields(nx, ny, nz, pr.fields()["h_eff"])
    M = _grid_fields(nx, ny, nz, m)
    ddx = (np.roll(M, -1, axis=3) - np.roll(M, 1, axis=3)) / (2 * d[0])
    ddy = (np.roll(M, -1, axis=2) - np.roll(M, 1, axis=2)) / (2 * d[1])
    pf = 2 * D / (MU0 * MS)
    want = np.stack([pf * ddx[2], pf * ddy[2], -pf * (ddx[0] + ddy[1])])
    assert np.allclose(h, want, rtol=1e-12, atol=1e-9 * np.abs(want).max())


def test_periodic_zhang_li_upwind_wraps(oracle):
    # the upwind derivative D = (u . grad) m takes the wrapped neighbour on a periodic axis
    # (zhang_li_stt_torque, fdm_fields.rs:1253-1340); with every field off the right-hand
    # side is the torque -m x (m x D) - beta m x D alone
    nx, ny, nz, d = 7, 4, 3, (2e-9, 3e-9, 2.5e-9)
    n = nx * ny * nz
    m = random_unit(n, 23)
    j, P, beta = (3e11, -2e11, 1e11), 0.6, 0.05
    pr = oracle.Problem(nx=nx, ny=ny, nz=nz, dx=d[0], dy=d[1], dz=d[2], ms=MS, a_ex=A, alpha=0.5, m0=m,
                        enable_exchange=False, enable_demag=False, current_density=j, stt_degree=P,
                        stt_beta=beta, periodic=(1, 0, 1))
    rhs = _grid_fields(nx, ny, nz, pr.fields()["rhs"])
    M = _grid_fields(nx, ny, nz, m)
    mu_b, e = 9.274009994e-24, 1.60217662e-19
    b = P * mu_b / (e * MS * (1 + beta * beta))
    u = [b * jj for jj in j]
    Dv = np.zeros_like(M)
    for a, (ax, per) in enumerate(((3, True), (2, False), (1, True))):
        step = d[a]
        if u[a] > 0:
            prev = np.roll(M, 1, axis=ax)
            diff = (M - prev) / step
            if not per:  # open axis: no upwind neighbour at the first cell
                idx = [slice(None)] * 4
                idx[ax] = 0
                diff[tuple(idx)] = 0.0
        else:
            nxt = np.roll(M, -1, axis=ax)
            diff = (nxt - M) / step
            if not per:
                idx = [slice(None)] * 4
                idx[ax] = -1
                diff[tuple(idx)] = 0.0
        Dv += u[a] * diff
    mm = M.reshape(3, -1).T
    DD = Dv.reshape(3, -1).T
    c1 = np.cross(mm, DD)
    c2 = np.cross(mm, c1)
    want = (-c2 - beta * c1).T.reshape(M.shape)
    assert np.allclose(rhs, want, rtol=1e-11, atol=1e-9 * np.abs(want).max())
