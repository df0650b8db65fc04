"""Engine-level known answers restated from crates/fullmag-engine/src/lib.rs:138-571,
crates/fullmag-engine/tests/physics_guardrails.rs and native/backends/fdm/tests/exchange_fp64_parity.cu."""
import numpy as np

from helpers import MU0, problem, random_unit


def test_uniform_state_has_zero_exchange(oracle):
    m = np.tile([0.6, 0.0, 0.8], (4 * 3 * 2, 1))
    pr = oracle.Problem(nx=4, ny=3, nz=2, dx=2e-9, dy=2e-9, dz=2e-9, ms=8e5, a_ex=1.3e-11, alpha=0.1,
                        enable_demag=False, m0=m)
    assert np.abs(pr.fields()["h_ex"]).max() < 1e-9


def test_flipped_centre_three_cells(oracle):
    """3x1x1 chain with the centre flipped: H_ex(centre) = 2A/(mu0 Ms) * 2 (m_side - m_c)/dx^2."""
    a, ms, dx = 1.3e-11, 8e5, 2e-9
    m = np.array([[1.0, 0, 0], [-1.0, 0, 0], [1.0, 0, 0]])
    pr = oracle.Problem(nx=3, ny=1, nz=1, dx=dx, dy=dx, dz=dx, ms=ms, a_ex=a, alpha=0.1, enable_demag=False, m0=m)
    h = pr.fields()["h_ex"]
    pref = 2 * a / (MU0 * ms)
    assert np.isclose(h[1, 0], pref * 4.0 / dx**2, rtol=1e-12)
    assert np.isclose(h[0, 0], pref * -2.0 / dx**2, rtol=1e-12)


def test_masked_cells_carry_no_field(oracle):
    kw = problem(5, 4, 2, seed=3)
    mask = np.ones(40, dtype=np.uint8)
    mask[[0, 7, 13, 22]] = 0
    pr = oracle.Problem(**kw, active_mask=mask)
    f = pr.fields()
    for k in ("h_ex", "h_demag", "h_eff", "rhs"):
        assert np.abs(f[k][mask == 0]).max() == 0.0


def test_exchange_energy_pair_and_field_forms_agree(oracle):
    pr = oracle.Problem(**problem(6, 5, 3, seed=4))
    st = pr.observe()
    assert np.isclose(st["e_exchange"], st["e_exchange_field"], rtol=1e-10)


def test_heun_preserves_norm_and_damping_lowers_energy(oracle):
    pr = oracle.Problem(**problem(8, 8, 2, seed=5, alpha=1.0, b_mt=None), integrator=oracle.HEUN)
    e0 = pr.observe()["e_total"]
    for _ in range(20):
        st = pr.step(2e-14)
    assert np.abs(np.linalg.norm(pr.get_m(), axis=1) - 1).max() < 1e-12
    assert st["e_total"] < e0


def test_damping_only_rhs_has_no_precession(oracle):
    kw = problem(4, 4, 1, seed=6)
    pr = oracle.Problem(**kw, disable_precession=True)
    f = pr.fields()
    m, h, k = f["rhs"] * 0 + kw["m0"], f["h_eff"], f["rhs"]
    # pure damping: k is parallel to m x (m x H)
    d = np.cross(m, np.cross(m, h))
    cr = np.cross(k, d)
    assert np.abs(cr).max() <= 1e-9 * np.abs(k).max() * np.abs(d).max()


def test_rk45_tracks_heun(oracle):
    kw = problem(6, 6, 1, seed=8, alpha=0.3)
    a = oracle.Problem(**kw, integrator=oracle.HEUN)
    b = oracle.Problem(**kw, integrator=oracle.DP45, max_error=1e-7)
    t = 0.0
    while t < 2e-12 - 1e-20:
        st = b.step(min(2e-14, 2e-12 - t))
        t += st["dt_used"]
    for _ in range(400):
        a.step(5e-15)
    assert np.abs(a.get_m() - b.get_m()).max() < 1e-3


def test_tangent_rk4_matches_central_differences(oracle):
    """The FP64 tangent-linear RK4 (checker of the engine's adjoint) against central
    differences of full RK4 runs: second-order convergence to the tangent."""
    nx, ny, n, dt, steps = 8, 4, 32, 5e-14, 40
    rng = np.random.default_rng(0)
    m0 = np.tile([1.0, 0.1, 0.0], (n, 1)) + 0.05 * rng.normal(size=(n, 3))
    m0 /= np.linalg.norm(m0, axis=1, keepdims=True)
    kw = problem(nx, ny, 1, alpha=0.05, b_mt=(5.0, 0.0, 0.0), ku1=1e4, u_axis=(1.0, 0.0, 0.0))
    kw["m0"] = m0
    hmap = rng.normal(0.0, 2e-3 / MU0, size=(n, 3))
    dh, dm0 = rng.normal(size=(n, 3)), 0.1 * rng.normal(size=(n, 3))

    def run(eps):
        pr = oracle.Problem(**kw, integrator=oracle.RK4)
        pr.set_field_map(hmap + eps * dh)
        pr.set_m(m0 + eps * dm0)
        for _ in range(steps):
            pr.step(dt)
        return pr.get_m()

    pr = oracle.Problem(**kw, integrator=oracle.RK4)
    pr.set_field_map(hmap)
    tl = pr.tangent_rk4(dt, steps, dh=dh, dm0=dm0)
    assert np.abs(pr.get_m() - run(0.0)).max() < 1e-14
    errs = [np.abs((run(e) - run(-e)) / (2 * e) - tl).max() / np.abs(tl).max() for e in (1e-1, 1e-2)]
    assert errs[1] < 1e-4 and errs[1] < errs[0] / 50
